// compat_driver.cu -- a reference-style caller of the drop-in header
// include/edge_loops.hpp: containers with the reference's member names
// (csr_t: rows, cols, nnzs, offsets, indices, values; matrix_t: rows, cols,
// m_data_ptr) held in thrust device vectors, and the reference's calls.
//
//   compat_driver <in.bin> <out.bin>
// in.bin: int64 rows, cols, nnz; int32 offsets[rows+1]; int32 indices[nnz];
//         float values[nnz]; int64 xlen; float x[xlen]
// out.bin: float y[5][rows] (merge_path_flat, thread_mapped, group_mapped,
//          work_oriented, original), then float C[rows][3] (spmm, B = x
//          repeated in 3 columns scaled by 1, 2, 3)
#include <edge_loops.hpp>
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>

#include <cstdio>
#include <vector>

struct csr_like {
  std::size_t rows, cols, nnzs;
  thrust::device_vector<int> offsets, indices;
  thrust::device_vector<float> values;
};

struct matrix_like {
  std::size_t rows, cols;
  thrust::device_vector<float> m_data;
  float* m_data_ptr;
};

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  long long hdr[3];
  if (std::fread(hdr, 8, 3, f) != 3) return 4;
  csr_like csr;
  csr.rows = hdr[0];
  csr.cols = hdr[1];
  csr.nnzs = hdr[2];
  std::vector<int> off(csr.rows + 1), idx(csr.nnzs);
  std::vector<float> val(csr.nnzs);
  long long xlen = 0;
  if (std::fread(off.data(), 4, off.size(), f) != off.size()) return 5;
  if (std::fread(idx.data(), 4, idx.size(), f) != idx.size()) return 5;
  if (std::fread(val.data(), 4, val.size(), f) != val.size()) return 5;
  if (std::fread(&xlen, 8, 1, f) != 1) return 5;
  std::vector<float> xh(xlen);
  if (std::fread(xh.data(), 4, xlen, f) != (size_t)xlen) return 5;
  std::fclose(f);
  csr.offsets = off;
  csr.indices = idx;
  csr.values = val;
  thrust::device_vector<float> x(xh.begin(), xh.end()), y(csr.rows);

  std::vector<float> out;
  auto grab = [&]() {
    thrust::host_vector<float> h = y;
    out.insert(out.end(), h.begin(), h.end());
    thrust::fill(y.begin(), y.end(), -1.0f);
  };
  try {
    auto t = loops::algorithms::spmv::merge_path_flat(csr, x, y);
    std::printf("merge_path_flat %.4f ms\n", t.milliseconds());
    grab();
    loops::algorithms::spmv::thread_mapped(csr, x, y);
    grab();
    loops::algorithms::spmv::group_mapped(csr, x, y);
    grab();
    loops::algorithms::spmv::work_oriented(csr, x, y);
    grab();
    loops::algorithms::spmv::original(csr, x, y);
    grab();
    matrix_like B{csr.cols, 3, {}, nullptr}, C{csr.rows, 3, {}, nullptr};
    std::vector<float> bh(csr.cols * 3);
    for (std::size_t r = 0; r < csr.cols; ++r)
      for (int c = 0; c < 3; ++c) bh[r * 3 + c] = xh[r] * (c + 1);
    B.m_data = bh;
    B.m_data_ptr = thrust::raw_pointer_cast(B.m_data.data());
    C.m_data.resize(csr.rows * 3);
    C.m_data_ptr = thrust::raw_pointer_cast(C.m_data.data());
    loops::algorithms::spmm::thread_mapped(csr, B, C);
    thrust::host_vector<float> ch = C.m_data;
    out.insert(out.end(), ch.begin(), ch.end());
  } catch (const edge_loops::exception_t& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 6;
  std::fwrite(out.data(), 4, out.size(), o);
  std::fclose(o);
  return 0;
}
