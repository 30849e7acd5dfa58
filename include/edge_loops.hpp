// edge_loops.hpp -- drop-in C++ entry points for the `loops` SpMV/SpMM path,
// implemented on the C ABI of edge_loops.h (link with libedgeloops.so).
//
// A program written against the reference replaces
//     #include <loops/algorithms/spmv/merge_path_flat.cuh>   (and friends)
// by
//     #include <edge_loops.hpp>
// and keeps its calls:
//     loops::algorithms::spmv::merge_path_flat(csr, x, y, stream);  // returns a timer
//     loops::algorithms::spmv::{thread_mapped,group_mapped,work_oriented,original}(csr, x, y, stream);
//     loops::algorithms::spmm::thread_mapped(csr, B, C, stream);
// [reference: include/loops/algorithms/spmv/*.cuh, spmm/thread_mapped.cuh]
//
// The containers stay the caller's: any csr type with members rows, cols,
// nnzs, offsets, indices, values (the reference's csr_t, container/csr.hxx:
// 32-95) whose vectors expose data() as a raw or thrust device pointer, any
// vector with data()/size(), and any dense matrix with rows, cols and
// m_data_ptr (the reference's matrix_t, container/matrix.cuh:8-51).
//
// Semantics kept from the reference: int32 offsets/indices, float/bf16/half
// values, the call synchronises `stream` before returning, merge_path_flat
// returns a timer whose milliseconds() covers the launch and that
// synchronisation.  Differences: y (C) is overwritten (equal to the
// reference's result on a zeroed y), and every failure throws
// edge_loops::exception_t (the reference throws only on allocation failure
// and leaves launch errors unchecked).
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>

#include "edge_loops.h"

namespace edge_loops {

struct exception_t : std::runtime_error {
  el_status status;
  exception_t(el_status s, const std::string& where)
      : std::runtime_error(where + ": " + el_status_string(s) + ": " +
                           el_last_error_string()),
        status(s) {}
};

inline void check(el_status s, const char* where) {
  if (s != EL_OK) throw exception_t(s, where);
}

// cudaEvent-based elapsed time, the shape of the reference's util::timer_t
// (util/timer.hxx:19-52).
struct timer_t {
  float elapsed = 0.f;
  float milliseconds() const { return elapsed; }
  float seconds() const { return elapsed * 1e-3f; }
};

namespace detail {

template <int N> struct rank : rank<N - 1> {};
template <> struct rank<0> {};

// thrust vectors: data() is a device_ptr with get()
template <class V>
auto raw(V& v, rank<2>) -> decltype(v.data().get()) { return v.data().get(); }
// raw-pointer containers
template <class V>
auto raw(V& v, rank<1>) -> decltype(&*v.data()) { return &*v.data(); }
template <class V>
auto raw(V& v) -> decltype(raw(v, rank<2>{})) { return raw(v, rank<2>{}); }

template <class T> struct dtype_of;
template <> struct dtype_of<float> { static constexpr int value = EL_F32; };
template <> struct dtype_of<const float> { static constexpr int value = EL_F32; };
#if defined(__CUDA_BF16_TYPES_EXIST__) || defined(__CUDA_BF16_H__)
template <> struct dtype_of<__nv_bfloat16> { static constexpr int value = EL_BF16; };
template <> struct dtype_of<const __nv_bfloat16> { static constexpr int value = EL_BF16; };
#endif
#if defined(__CUDA_FP16_TYPES_EXIST__) || defined(__CUDA_FP16_H__)
template <> struct dtype_of<__half> { static constexpr int value = EL_F16; };
template <> struct dtype_of<const __half> { static constexpr int value = EL_F16; };
#endif

template <class Csr>
el_csr as_el(Csr& csr) {
  static_assert(sizeof(*raw(csr.offsets)) == 4 && sizeof(*raw(csr.indices)) == 4,
                "int32 offsets and indices");
  using VT = typename std::remove_reference<decltype(*raw(csr.values))>::type;
  el_csr a{};
  a.rows = (int64_t)csr.rows;
  a.cols = (int64_t)csr.cols;
  a.nnz = (int64_t)csr.nnzs;
  a.offsets = reinterpret_cast<const int32_t*>(raw(csr.offsets));
  a.indices = reinterpret_cast<const int32_t*>(raw(csr.indices));
  a.values = raw(csr.values);
  a.value_dtype = dtype_of<VT>::value;
  a.row_scale = nullptr;
  return a;
}

template <class Csr, class Vec>
void spmv(int32_t schedule, Csr& csr, Vec& x, Vec& y, cudaStream_t stream,
          const el_spmv_opts* opts = nullptr) {
  el_csr a = as_el(csr);
  const float* xp = raw(x);
  float* yp = raw(y);
  check(el_spmv(nullptr, &a, schedule, opts, xp, yp, (el_stream_t)stream), "el_spmv");
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) throw exception_t(EL_ERR_CUDA, cudaGetErrorString(e));
  uint32_t flags = 0;
  check(el_workspace_errors(nullptr, (el_stream_t)stream, &flags, 1), "el_workspace_errors");
  if (flags) throw exception_t(EL_ERR_DEVICE, "device flags " + std::to_string(flags));
}

}  // namespace detail
}  // namespace edge_loops

namespace loops {
namespace algorithms {
namespace spmv {

// [include/loops/algorithms/spmv/merge_path_flat.cuh:96-139]
template <class Csr, class Vec>
edge_loops::timer_t merge_path_flat(Csr& csr, Vec& x, Vec& y, cudaStream_t stream = 0) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, stream);
  edge_loops::detail::spmv(EL_SCHED_MERGE_PATH_FLAT, csr, x, y, stream);
  cudaEventRecord(b, stream);
  cudaEventSynchronize(b);
  edge_loops::timer_t t;
  cudaEventElapsedTime(&t.elapsed, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return t;
}

// [include/loops/algorithms/spmv/thread_mapped.cuh:68-91]
template <class Csr, class Vec>
void thread_mapped(Csr& csr, Vec& x, Vec& y, cudaStream_t stream = 0) {
  edge_loops::detail::spmv(EL_SCHED_THREAD_MAPPED, csr, x, y, stream);
}

// [include/loops/algorithms/spmv/original.cuh:59-76] (one row per thread:
// the thread_mapped schedule with one thread per row)
template <class Csr, class Vec>
void original(Csr& csr, Vec& x, Vec& y, cudaStream_t stream = 0) {
  edge_loops::detail::spmv(EL_SCHED_THREAD_MAPPED, csr, x, y, stream);
}

// [include/loops/algorithms/spmv/group_mapped.cuh:73-105]
template <class Csr, class Vec>
void group_mapped(Csr& csr, Vec& x, Vec& y, cudaStream_t stream = 0) {
  edge_loops::detail::spmv(EL_SCHED_GROUP_MAPPED, csr, x, y, stream);
}

// [include/loops/algorithms/spmv/work_oriented.cuh:88-111]
template <class Csr, class Vec>
void work_oriented(Csr& csr, Vec& x, Vec& y, cudaStream_t stream = 0) {
  edge_loops::detail::spmv(EL_SCHED_WORK_ORIENTED, csr, x, y, stream);
}

}  // namespace spmv

namespace spmm {

// [include/loops/algorithms/spmm/thread_mapped.cuh:67-90]
template <class Csr, class Mat>
void thread_mapped(Csr& csr, Mat& B, Mat& C, cudaStream_t stream = 0) {
  el_csr a = edge_loops::detail::as_el(csr);
  using BT = typename std::remove_reference<decltype(*B.m_data_ptr)>::type;
  edge_loops::check(
      el_spmm(nullptr, &a, EL_SCHED_THREAD_MAPPED, nullptr, B.m_data_ptr,
              edge_loops::detail::dtype_of<BT>::value, (int64_t)B.cols, (int64_t)B.cols,
              C.m_data_ptr, (int64_t)C.cols, (el_stream_t)stream),
      "el_spmm");
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) throw edge_loops::exception_t(EL_ERR_CUDA, cudaGetErrorString(e));
}

}  // namespace spmm
}  // namespace algorithms
}  // namespace loops
