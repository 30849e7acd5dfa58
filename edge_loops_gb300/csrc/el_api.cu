// el_api.cu -- the C ABI declared in include/edge_loops.h: argument checks,
// workspaces, and dispatch to the schedule launchers.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "el_internal.h"

// --------------------------------------------------------------- workspace
struct el_workspace {
  int device;
  void* dev;  // WsHeader + CarrySlot[nslots]
  long long nslots;
  void* scratch;  // row-vector carries of the merge-path SpMM
  size_t scratch_bytes;
  // el_spmv_host: device staging memory, a copy stream and its events
  void* stage = nullptr;
  size_t stage_bytes = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t events[4] = {nullptr, nullptr, nullptr, nullptr};
};

namespace el {

namespace {
thread_local std::string g_last_error;
thread_local long long* g_trace = nullptr;  // el_debug_range_trace
thread_local long long g_trace_cap = 0;
std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, el_workspace*> g_default_ws;
std::map<int, DeviceInfo> g_dev_info;
std::map<std::pair<const void*, long long>, int> g_occupancy;

constexpr long long kInitialSlots = 8192;
constexpr unsigned long long kDefaultWaitNs = 2000000000ull;  // 2 s
}  // namespace

el_status fail(el_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

el_status cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return EL_OK;
  if (e == cudaErrorMemoryAllocation)
    return fail(EL_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(EL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void range_trace(long long** buf, long long* cap) {
  *buf = g_trace;
  *cap = g_trace ? g_trace_cap : 0;
}

const DeviceInfo& device_info(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_dev_info.find(device);
  if (it != g_dev_info.end()) return it->second;
  DeviceInfo d{1, 48 * 1024};
  cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&d.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                         device);
  return g_dev_info.emplace(device, d).first->second;
}

int resident_ctas_per_sm(const void* kernel, int threads, size_t smem) {
  int dev = 0;
  cudaGetDevice(&dev);
  const long long key2 = ((long long)dev << 48) ^ ((long long)threads << 32) ^ (long long)smem;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_occupancy.find({kernel, key2});
    if (it != g_occupancy.end()) return it->second;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) !=
      cudaSuccess)
    n = 0;
  std::lock_guard<std::mutex> lk(g_mu);
  g_occupancy[{kernel, key2}] = n;
  return n;
}

namespace {

el_status ws_alloc(el_workspace* ws, long long nslots) {
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != ws->device) cudaSetDevice(ws->device);
  const size_t bytes = sizeof(WsHeader) + (size_t)nslots * sizeof(CarrySlot);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e == cudaSuccess) e = cudaMemset(p, 0, bytes);
  if (cur != ws->device) cudaSetDevice(cur);
  if (e != cudaSuccess) {
    if (p) cudaFree(p);
    return cuda_status(e, "workspace allocation");
  }
  ws->dev = p;
  ws->nslots = nslots;
  return EL_OK;
}

// Makes sure `ws` has at least `need` carry slots.  Growing waits for the
// device (cudaFree synchronises), so size workspaces before graph capture.
el_status ws_reserve(el_workspace* ws, long long need) {
  if (need <= ws->nslots) return EL_OK;
  long long n = ws->nslots * 2;
  if (n < need) n = need;
  void* old = ws->dev;
  el_status s = ws_alloc(ws, n);
  if (s != EL_OK) return s;
  if (old) cudaFree(old);
  return EL_OK;
}

// Makes sure `ws` has `bytes` of scratch (same caveat as ws_reserve).
el_status ws_reserve_scratch(el_workspace* ws, size_t bytes) {
  if (bytes <= ws->scratch_bytes) return EL_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != ws->device) cudaSetDevice(ws->device);
  if (ws->scratch) cudaFree(ws->scratch);
  ws->scratch = nullptr;
  ws->scratch_bytes = 0;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (cur != ws->device) cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_status(e, "workspace scratch allocation");
  ws->scratch = p;
  ws->scratch_bytes = bytes;
  return EL_OK;
}

WsView ws_view(el_workspace* ws) {
  WsView v;
  v.hdr = reinterpret_cast<WsHeader*>(ws->dev);
  v.slots = reinterpret_cast<CarrySlot*>(reinterpret_cast<char*>(ws->dev) +
                                         sizeof(WsHeader));
  v.nslots = ws->nslots;
  return v;
}

el_status default_ws(int device, cudaStream_t stream, el_workspace** out) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_default_ws.find({device, stream});
    if (it != g_default_ws.end()) {
      *out = it->second;
      return EL_OK;
    }
  }
  el_workspace* ws = new el_workspace{device, nullptr, 0, nullptr, 0};
  el_status s = ws_alloc(ws, kInitialSlots);
  if (s != EL_OK) {
    delete ws;
    return s;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  auto ins = g_default_ws.emplace(std::make_pair(device, stream), ws);
  if (!ins.second) {  // another thread won the race
    cudaFree(ws->dev);
    delete ws;
  }
  *out = ins.first->second;
  return EL_OK;
}

el_status check_csr(const el_csr* A) {
  if (!A) return fail(EL_ERR_NULL_POINTER, "A is NULL");
  if (A->rows < 0 || A->cols < 0 || A->nnz < 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "negative size (rows=%lld cols=%lld nnz=%lld)",
                (long long)A->rows, (long long)A->cols, (long long)A->nnz);
  if (A->rows + A->nnz >= kMergeLimit || A->cols >= (1LL << 31))
    return fail(EL_ERR_OVERFLOW,
                "rows+nnz = %lld needs 64-bit merge coordinates (limit 2^31 - 2^16: the "
                "reference's int32 search, less headroom for tile arithmetic)",
                (long long)(A->rows + A->nnz));
  if (A->value_dtype < EL_F32 || A->value_dtype > EL_F16)
    return fail(EL_ERR_INVALID_ARGUMENT, "unknown value dtype %d", A->value_dtype);
  if (A->rows > 0 && !A->offsets) return fail(EL_ERR_NULL_POINTER, "offsets is NULL");
  if (A->nnz > 0 && (!A->indices || !A->values))
    return fail(EL_ERR_NULL_POINTER, "indices/values is NULL");
  return EL_OK;
}

el_status resolve_ws(el_workspace* ws, cudaStream_t stream, int device,
                     el_workspace** out) {
  if (ws) {
    if (ws->device != device)
      return fail(EL_ERR_INVALID_ARGUMENT, "workspace belongs to device %d, current is %d",
                  ws->device, device);
    *out = ws;
    return EL_OK;
  }
  return default_ws(device, stream, out);
}

}  // namespace

WsView workspace_view(el_workspace* ws) { return ws_view(ws); }

el_status workspace_resolve(el_workspace* ws, cudaStream_t stream, int device,
                            el_workspace** out) {
  return resolve_ws(ws, stream, device, out);
}

el_status workspace_stage(el_workspace* ws, size_t bytes, void** stage,
                          cudaStream_t* copy_stream, cudaEvent_t* events) {
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != ws->device) return fail(EL_ERR_INVALID_ARGUMENT, "workspace of another device");
  cudaError_t e = cudaSuccess;
  if (!ws->copy_stream) {
    e = cudaStreamCreateWithFlags(&ws->copy_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e, "copy stream");
    for (int i = 0; i < 4 && e == cudaSuccess; ++i)
      e = cudaEventCreateWithFlags(&ws->events[i], cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_status(e, "copy events");
  }
  if (bytes > ws->stage_bytes) {
    if (ws->stage) cudaFree(ws->stage);  // waits for the device
    ws->stage = nullptr;
    ws->stage_bytes = 0;
    e = cudaMalloc(&ws->stage, bytes);
    if (e != cudaSuccess) return cuda_status(e, "staging memory");
    ws->stage_bytes = bytes;
  }
  *stage = ws->stage;
  *copy_stream = ws->copy_stream;
  for (int i = 0; i < 4; ++i) events[i] = ws->events[i];
  return EL_OK;
}

el_status workspace_prepare(el_workspace* ws, const el_csr& A, int schedule) {
  SpmvCall c;
  c.A = A;
  c.x = nullptr;
  c.y = nullptr;
  el_spmv_opts_default(&c.o);
  c.stream = nullptr;
  c.wait_ns = kDefaultWaitNs;
  c.device = ws->device;
  c.ws = ws_view(ws);
  if (schedule == EL_SCHED_MERGE_PATH_FLAT) return ws_reserve(ws, merge_path_slots_needed(c));
  if (schedule == EL_SCHED_WORK_ORIENTED) return ws_reserve(ws, work_oriented_slots_needed(c));
  return EL_OK;
}

}  // namespace el

using namespace el;

extern "C" {

int el_version(void) { return EL_VERSION; }

const char* el_status_string(el_status s) {
  switch (s) {
    case EL_OK: return "EL_OK";
    case EL_ERR_INVALID_ARGUMENT: return "EL_ERR_INVALID_ARGUMENT";
    case EL_ERR_NULL_POINTER: return "EL_ERR_NULL_POINTER";
    case EL_ERR_OVERFLOW: return "EL_ERR_OVERFLOW";
    case EL_ERR_UNSUPPORTED: return "EL_ERR_UNSUPPORTED";
    case EL_ERR_MALFORMED_CSR: return "EL_ERR_MALFORMED_CSR";
    case EL_ERR_CUDA: return "EL_ERR_CUDA";
    case EL_ERR_OUT_OF_MEMORY: return "EL_ERR_OUT_OF_MEMORY";
    case EL_ERR_DEVICE: return "EL_ERR_DEVICE";
    case EL_ERR_IO: return "EL_ERR_IO";
    case EL_ERR_PARSE: return "EL_ERR_PARSE";
  }
  return "EL_ERR_UNKNOWN";
}

const char* el_last_error_string(void) { return g_last_error.c_str(); }

el_status el_debug_range_trace(int64_t* ranges, int64_t capacity) {
  if (ranges && capacity <= 0) return fail(EL_ERR_INVALID_ARGUMENT, "capacity must be > 0");
  g_trace = reinterpret_cast<long long*>(ranges);
  g_trace_cap = ranges ? capacity : 0;
  return EL_OK;
}

void el_spmv_opts_default(el_spmv_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
}

el_status el_workspace_create(int device, el_workspace** out) {
  if (!out) return fail(EL_ERR_NULL_POINTER, "out is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDeviceCount");
  if (device < 0 || device >= n) return fail(EL_ERR_INVALID_ARGUMENT, "no device %d", device);
  el_workspace* ws = new el_workspace{device, nullptr, 0, nullptr, 0};
  el_status s = ws_alloc(ws, kInitialSlots);
  if (s != EL_OK) {
    delete ws;
    return s;
  }
  *out = ws;
  return EL_OK;
}

el_status el_workspace_destroy(el_workspace* ws) {
  if (!ws) return EL_OK;
  if (ws->dev) cudaFree(ws->dev);
  if (ws->scratch) cudaFree(ws->scratch);
  if (ws->stage) cudaFree(ws->stage);
  for (int i = 0; i < 4; ++i)
    if (ws->events[i]) cudaEventDestroy(ws->events[i]);
  if (ws->copy_stream) cudaStreamDestroy(ws->copy_stream);
  delete ws;
  return EL_OK;
}

el_status el_workspace_errors(el_workspace* ws, el_stream_t stream,
                              uint32_t* flags, int clear) {
  if (!flags) return fail(EL_ERR_NULL_POINTER, "flags is NULL");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  el_workspace* w = nullptr;
  el_status s = resolve_ws(ws, (cudaStream_t)stream, dev, &w);
  if (s != EL_OK) return s;
  WsView v = ws_view(w);
  e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
  unsigned h = 0;
  e = cudaMemcpy(&h, &v.hdr->errors, sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e, "reading device flags");
  *flags = h;
  if (clear && h) {
    e = cudaMemset(&v.hdr->errors, 0, 2 * sizeof(unsigned));
    if (e != cudaSuccess) return cuda_status(e, "clearing device flags");
  }
  return EL_OK;
}

el_status el_spmv(el_workspace* ws, const el_csr* A, int32_t schedule,
                  const el_spmv_opts* opts, const float* x, float* y,
                  el_stream_t stream) {
  el_status s = check_csr(A);
  if (s != EL_OK) return s;
  if (A->rows > 0 && !y) return fail(EL_ERR_NULL_POINTER, "y is NULL");
  if (A->nnz > 0 && !x) return fail(EL_ERR_NULL_POINTER, "x is NULL");
  if (schedule == EL_SCHED_BUCKETING)
    return fail(EL_ERR_UNSUPPORTED,
                "the bucketing schedule is declared by loops but never implemented");
  if (schedule < EL_SCHED_MERGE_PATH_FLAT || schedule > EL_SCHED_AUTO)
    return fail(EL_ERR_INVALID_ARGUMENT, "unknown schedule %d", schedule);
  SpmvCall c;
  c.A = *A;
  c.x = x;
  c.y = y;
  el_spmv_opts_default(&c.o);
  if (opts) c.o = *opts;
  c.stream = (cudaStream_t)stream;
  c.wait_ns = c.o.wait_limit_us > 0 ? (unsigned long long)c.o.wait_limit_us * 1000ull
                                     : kDefaultWaitNs;
  range_trace(&c.trace, &c.trace_cap);
  cudaError_t e = cudaGetDevice(&c.device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (A->rows == 0) return EL_OK;
  el_workspace* w = nullptr;
  s = resolve_ws(ws, c.stream, c.device, &w);
  if (s != EL_OK) return s;
  if (schedule == EL_SCHED_AUTO) {
    // the selection cost model with the longest row assumed to hold every
    // nonzero (nothing else is known without a synchronisation): merge_path
    // unless the matrix is so small that even then thread_mapped is faster
    int32_t sched = EL_SCHED_MERGE_PATH_FLAT, tpr = 0;
    s = el_select_schedule(A->rows, A->cols, A->nnz, A->nnz, &sched, &tpr, nullptr);
    if (s != EL_OK) return s;
    schedule = sched;
    if (schedule == EL_SCHED_THREAD_MAPPED) c.o.threads_per_row = tpr;
  }
  switch (schedule) {
    case EL_SCHED_MERGE_PATH_FLAT: {
      c.ws = ws_view(w);
      s = ws_reserve(w, merge_path_slots_needed(c));
      if (s != EL_OK) return s;
      c.ws = ws_view(w);
      return launch_merge_path(c);
    }
    case EL_SCHED_WORK_ORIENTED: {
      c.ws = ws_view(w);
      s = ws_reserve(w, work_oriented_slots_needed(c));
      if (s != EL_OK) return s;
      c.ws = ws_view(w);
      return launch_work_oriented(c);
    }
    case EL_SCHED_THREAD_MAPPED:
      c.ws = ws_view(w);
      return launch_thread_mapped(c);
    case EL_SCHED_GROUP_MAPPED:
      c.ws = ws_view(w);
      return launch_group_mapped(c);
  }
  return fail(EL_ERR_INVALID_ARGUMENT, "unknown schedule %d", schedule);
}

el_status el_spmm(el_workspace* ws, const el_csr* A, int32_t schedule,
                  const el_spmv_opts* opts, const void* B, int32_t b_dtype,
                  int64_t n, int64_t ldb, float* C, int64_t ldc,
                  el_stream_t stream) {
  el_status s = check_csr(A);
  if (s != EL_OK) return s;
  if (n < 0) return fail(EL_ERR_INVALID_ARGUMENT, "n < 0");
  if (ldb < n || ldc < n) return fail(EL_ERR_INVALID_ARGUMENT, "ldb/ldc smaller than n");
  if (b_dtype < EL_F32 || b_dtype > EL_F16)
    return fail(EL_ERR_INVALID_ARGUMENT, "unknown B dtype %d", b_dtype);
  if (A->rows > 0 && n > 0 && !C) return fail(EL_ERR_NULL_POINTER, "C is NULL");
  if (A->nnz > 0 && n > 0 && !B) return fail(EL_ERR_NULL_POINTER, "B is NULL");
  if (schedule == EL_SCHED_BUCKETING || schedule == EL_SCHED_WORK_ORIENTED)
    return fail(EL_ERR_UNSUPPORTED, "SpMM schedules: thread_mapped, group_mapped, merge_path");
  if (schedule < EL_SCHED_MERGE_PATH_FLAT || schedule > EL_SCHED_AUTO)
    return fail(EL_ERR_INVALID_ARGUMENT, "unknown schedule %d", schedule);
  SpmmCall c;
  c.A = *A;
  c.B = B;
  c.b_dtype = b_dtype;
  c.n = n;
  c.ldb = ldb;
  c.ldc = ldc;
  c.C = C;
  el_spmv_opts_default(&c.o);
  if (opts) c.o = *opts;
  c.stream = (cudaStream_t)stream;
  c.wait_ns = c.o.wait_limit_us > 0 ? (unsigned long long)c.o.wait_limit_us * 1000ull
                                     : kDefaultWaitNs;
  c.scratch = nullptr;
  c.scratch_bytes = 0;
  cudaError_t e = cudaGetDevice(&c.device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (A->rows == 0 || n == 0) return EL_OK;
  el_workspace* w = nullptr;
  s = resolve_ws(ws, c.stream, c.device, &w);
  if (s != EL_OK) return s;
  if (schedule == EL_SCHED_AUTO) schedule = EL_SCHED_MERGE_PATH_FLAT;
  s = ws_reserve(w, spmm_slots_needed(c, schedule));
  if (s != EL_OK) return s;
  s = ws_reserve_scratch(w, spmm_scratch_bytes(c, schedule));
  if (s != EL_OK) return s;
  c.ws = ws_view(w);
  c.scratch = w->scratch;
  c.scratch_bytes = w->scratch_bytes;
  return launch_spmm(c, schedule);
}

el_status el_csr_validate(const el_csr* A, el_stream_t stream, uint32_t* flags) {
  el_status s = check_csr(A);
  if (s != EL_OK) return s;
  if (!flags) return fail(EL_ERR_NULL_POINTER, "flags is NULL");
  *flags = 0;
  if (A->rows == 0 && A->nnz == 0) return EL_OK;
  if (A->rows == 0) {
    *flags = EL_FLAG_NNZ_MISMATCH;
    return fail(EL_ERR_MALFORMED_CSR, "rows == 0 but nnz = %lld", (long long)A->nnz);
  }
  unsigned* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(unsigned));
  if (e != cudaSuccess) return cuda_status(e, "validate scratch");
  e = cudaMemsetAsync(d, 0, sizeof(unsigned), (cudaStream_t)stream);
  if (e == cudaSuccess) {
    s = launch_validate(*A, d, (cudaStream_t)stream);
    if (s != EL_OK) {
      cudaFree(d);
      return s;
    }
    unsigned h = 0;
    e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    *flags = h;
  }
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e, "validate");
  if (*flags) return fail(EL_ERR_MALFORMED_CSR, "CSR defects: flags 0x%x", *flags);
  return EL_OK;
}

int64_t el_merge_path_num_tiles(int64_t rows, int64_t nnz, int32_t tpb, int32_t ipt) {
  if (rows < 0 || nnz < 0 || tpb <= 0 || ipt <= 0) return -1;
  const long long items = (long long)tpb * ipt;
  return (rows + nnz + items - 1) / items;
}

el_status el_merge_path_partition(const int32_t* offsets, int64_t rows, int64_t nnz,
                                  int32_t tpb, int32_t ipt, uint32_t* coords,
                                  el_stream_t stream) {
  if (rows < 0 || nnz < 0 || tpb <= 0 || ipt <= 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "bad partition arguments");
  if (rows + nnz >= kMergeLimit) return fail(EL_ERR_OVERFLOW, "rows+nnz >= 2^31 - 2^16");
  if (rows == 0) return fail(EL_ERR_INVALID_ARGUMENT, "rows == 0");
  if (!offsets || !coords) return fail(EL_ERR_NULL_POINTER, "offsets/coords is NULL");
  return launch_partition_tiles(offsets, rows, nnz, (int64_t)tpb * ipt, coords,
                                (cudaStream_t)stream);
}

el_status el_merge_path_thread_coords(const int32_t* offsets, int64_t rows, int64_t nnz,
                                      int32_t tpb, int32_t ipt, uint32_t* coords,
                                      el_stream_t stream) {
  if (rows <= 0 || nnz < 0 || tpb < 2 || tpb > 1024 || ipt <= 0 || ipt > 64)
    return fail(EL_ERR_INVALID_ARGUMENT, "bad partition arguments");
  if (rows + nnz >= kMergeLimit) return fail(EL_ERR_OVERFLOW, "rows+nnz >= 2^31 - 2^16");
  if (!offsets || !coords) return fail(EL_ERR_NULL_POINTER, "offsets/coords is NULL");
  return launch_partition_threads(offsets, rows, nnz, tpb, ipt, coords,
                                  (cudaStream_t)stream);
}

el_status el_work_oriented_partition(const int32_t* offsets, int64_t rows, int64_t nnz,
                                     int64_t num_threads, int64_t* coords,
                                     el_stream_t stream) {
  if (rows <= 0 || nnz < 0 || num_threads <= 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "bad partition arguments");
  if (rows + nnz >= kMergeLimit) return fail(EL_ERR_OVERFLOW, "rows+nnz >= 2^31 - 2^16");
  if (!offsets || !coords) return fail(EL_ERR_NULL_POINTER, "offsets/coords is NULL");
  return launch_partition_work_oriented(offsets, rows, nnz, num_threads, coords,
                                        (cudaStream_t)stream);
}

el_status el_quantize_values(const int32_t* offsets, int64_t rows, int64_t nnz,
                             const float* values, int32_t dtype, void* out_values,
                             float* row_scale, el_stream_t stream) {
  if (rows < 0 || nnz < 0) return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (dtype != EL_BF16 && dtype != EL_F16)
    return fail(EL_ERR_INVALID_ARGUMENT, "quantize dtype must be BF16 or FP16");
  if (rows == 0) return EL_OK;
  if (!offsets || (nnz > 0 && (!values || !out_values)))
    return fail(EL_ERR_NULL_POINTER, "NULL input");
  return launch_quantize(offsets, rows, nnz, values, dtype, out_values, row_scale,
                         (cudaStream_t)stream);
}

}  // extern "C"
