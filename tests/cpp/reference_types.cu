// reference_types.cu -- compile-only check that include/edge_loops.hpp
// accepts the reference's own containers (csr_t, vector_t, matrix_t from
// include/loops/container/) in place of its algorithm headers.
#include <loops/container/container.hxx>
#include <loops/container/csr.hxx>
#include <edge_loops.hpp>

using namespace loops;

float drop_in(csr_t<int, int, float>& csr, vector_t<float>& x, vector_t<float>& y,
              matrix_t<float>& B, matrix_t<float>& C) {
  auto t = algorithms::spmv::merge_path_flat(csr, x, y);
  algorithms::spmv::thread_mapped(csr, x, y);
  algorithms::spmv::group_mapped(csr, x, y);
  algorithms::spmv::work_oriented(csr, x, y);
  algorithms::spmv::original(csr, x, y);
  algorithms::spmm::thread_mapped(csr, B, C);
  return t.milliseconds();
}
