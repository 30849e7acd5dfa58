// ref_kernels.cu -- the reference's own SpMV kernels (merge_path_flat,
// thread_mapped, group_mapped, work_oriented, original) and its SpMM
// (thread_mapped), instantiated for
// int offsets and indices and float values exactly as the reference's
// launchers instantiate them (algorithms/spmv/*.cuh), so that they can be
// run on a GPU from a cubin (oracle/ref/ref_gpu.py) -- test infrastructure,
// never part of the product.
//
// build_ref.sh compiles this file twice:
//   -cubin  the kernels (device code only) -> oracle/_ref/ref_kernels.cubin;
//   host    a program that prints, as JSON, what a launcher needs and that
//           only the host compiler knows: the size of the merge-path
//           preprocess object passed by value, and the bytes of a
//           thread_mapped setup object and of a dense matrix_t built with
//           sentinel values (the launcher puts the real pointers and sizes
//           in their place).

// the headers the reference's example drivers include first
// (examples/spmv/helpers.hxx:14-22), on which the algorithm headers rely
#include <thrust/device_vector.h>
#include <loops/error.hxx>
#include <loops/container/formats.hxx>
#include <loops/container/vector.hxx>
#include <loops/memory.hxx>
#include <loops/util/device.hxx>
#include <loops/util/timer.hxx>

#include <loops/container/matrix.cuh>
#include <loops/algorithms/spmm/thread_mapped.cuh>
#include <loops/algorithms/spmv/group_mapped.cuh>
#include <loops/algorithms/spmv/merge_path_flat.cuh>
#include <loops/algorithms/spmv/original.cuh>
#include <loops/algorithms/spmv/thread_mapped.cuh>
#include <loops/algorithms/spmv/work_oriented.cuh>

#include <cstdint>
#include <cstdio>
#include <cstring>

namespace R = loops::algorithms::spmv;
namespace S = loops::schedule;

// merge_path_flat.cuh:113-114 and :131-133 (block 128, 5 items per thread)
using mp_meta_t = S::merge_path::preprocess_t<128, 5, int, int, std::size_t, std::size_t>;
// thread_mapped.cuh:79-80
using tm_setup_t = S::setup<S::algorithms_t::thread_mapped, 1, 1, int, int>;

template __global__ void R::__merge_path_flat<128, 5, mp_meta_t, int, int, float>(
    mp_meta_t, std::size_t, std::size_t, std::size_t, int*, int*, const float*, const float*,
    float*);
template __global__ void R::__thread_mapped<tm_setup_t, int, int, float>(
    tm_setup_t, const std::size_t, const std::size_t, const std::size_t, const int*, const int*,
    const float*, const float*, float*);
template __global__ void R::__group_mapped<128, int, int, float>(std::size_t, std::size_t,
                                                                  std::size_t, int*, int*,
                                                                  const float*, const float*,
                                                                  float*);
template __global__ void R::__work_oriented<128, int, int, float>(std::size_t, std::size_t,
                                                                   std::size_t, int*, int*,
                                                                   const float*, const float*,
                                                                   float*);
// algorithms/spmm/thread_mapped.cuh:67-86 (the reference's one SpMM)
template __global__ void loops::algorithms::spmm::__thread_mapped<tm_setup_t, int, int, float>(
    tm_setup_t, const std::size_t, const std::size_t, const std::size_t, const int*, const int*,
    const float*, const loops::matrix_t<float>, loops::matrix_t<float>);
template __global__ void R::__original<int, int, float>(const std::size_t, const std::size_t,
                                                        const std::size_t, const int*,
                                                        const int*, const float*, const float*,
                                                        float*);

#ifndef __CUDA_ARCH__
int main() {
  const std::uint64_t kPtr = 0xA1A1A1A1A1A1A1A1ull, kRows = 0xB2B2B2B2B2B2B2B2ull,
                      kNnz = 0xC3C3C3C3C3C3C3C3ull;
  tm_setup_t tm(reinterpret_cast<int*>(kPtr), (std::size_t)kRows, (std::size_t)kNnz);
  unsigned char bytes[sizeof(tm_setup_t)];
  std::memcpy(bytes, &tm, sizeof(tm));
  std::printf("{\"merge_path_meta_size\": %zu, \"merge_path_meta_align\": %zu, ",
              sizeof(mp_meta_t), alignof(mp_meta_t));
  std::printf("\"thread_mapped_setup_align\": %zu, \"thread_mapped_setup\": \"",
              alignof(tm_setup_t));
  for (size_t i = 0; i < sizeof(bytes); ++i) std::printf("%02x", bytes[i]);
  // a dense matrix_t passed by value: rows, cols and the data pointer (its
  // vector member is not copied by the copy constructor, nor read on the GPU)
  loops::matrix_t<float> mt;
  mt.rows = (std::size_t)kRows;
  mt.cols = (std::size_t)kNnz;
  mt.m_data_ptr = reinterpret_cast<float*>(kPtr);
  loops::matrix_t<float> mc(mt);
  unsigned char mb[sizeof(mc)];
  std::memcpy(mb, &mc, sizeof(mc));
  std::printf("\", \"matrix_align\": %zu, \"matrix\": \"", alignof(loops::matrix_t<float>));
  for (size_t i = 0; i < sizeof(mb); ++i) std::printf("%02x", mb[i]);
  std::printf("\", \"sentinels\": {\"offsets\": \"%016llx\", \"rows\": \"%016llx\", "
              "\"nnz\": \"%016llx\"}}\n",
              (unsigned long long)kPtr, (unsigned long long)kRows, (unsigned long long)kNnz);
  return 0;
}
#endif
