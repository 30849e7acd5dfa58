// device_api_driver.cu -- user kernels written with include/edge_loops_device.cuh
// (the load-balanced loop API), run on a CSR read from a file:
//   in : int64 rows, cols, nnz; int32 offsets[rows+1]; int32 indices[nnz];
//        float values[nnz]; int64 n; float x[n]
//   out: float y_merge[rows]   (merge-path ranges, partial rows by atomicAdd)
//        int32 count[rows]     (on_nonzero calls per row over all ranges)
//        int32 ends[rows]      (on_row_end calls per row over all ranges)
//        float y_rows[rows]    (thread-mapped loop, nonzero order, no FMA)
//        int32 mismatches      (warp_merge_path_search vs merge_path_search)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <edge_loops_device.cuh>

namespace eld = edge_loops::device;

#define CHECK(x)                                                              \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));          \
      std::exit(1);                                                           \
    }                                                                         \
  } while (0)

// y = A x with one merge range per thread: the rows closed inside a range
// and the open row at its end add their partial sums to y atomically
__global__ void spmv_ranges(const int* off, const int* idx, const float* val, const float* x,
                            float* y, int* count, int* ends, int rows, int nnz) {
  const long long parts = (long long)gridDim.x * blockDim.x;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  eld::coord b, e;
  eld::merge_path_range(off, rows, nnz, parts, p, b, e);
  float acc = 0.f;
  eld::for_each_in_range(
      off, b, e,
      [&](int row, int nz) {
        acc += val[nz] * x[idx[nz]];
        atomicAdd(count + row, 1);
      },
      [&](int row) {
        atomicAdd(y + row, acc);
        atomicAdd(ends + row, 1);
        acc = 0.f;
      });
  if (e.row < rows && acc != 0.f) atomicAdd(y + e.row, acc);  // the open row
}

__global__ void spmv_rows(const int* off, const int* idx, const float* val, const float* x,
                          float* y, int rows) {
  float acc = 0.f;
  eld::for_each_row(
      off, rows, [&](int, int nz) { acc = __fadd_rn(acc, __fmul_rn(val[nz], x[idx[nz]])); },
      [&](int row) {
        y[row] = acc;
        acc = 0.f;
      });
}

__global__ void check_warp_search(const int* off, int rows, int nnz, int* mismatches) {
  const long long total = (long long)rows + nnz;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long d = warp; d <= total; d += warps) {  // warp-uniform
    const eld::coord a = eld::warp_merge_path_search(off, rows, nnz, d);
    const eld::coord s = eld::merge_path_search(off, rows, nnz, d);
    if ((threadIdx.x & 31) == 0 && (a.row != s.row || a.nz != s.nz)) atomicAdd(mismatches, 1);
  }
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 1;
  long long hdr[3], n = 0;
  if (std::fread(hdr, 8, 3, f) != 3) return 1;
  const int rows = (int)hdr[0], nnz = (int)hdr[2];
  std::vector<int> off(rows + 1), idx(nnz > 0 ? nnz : 1);
  std::vector<float> val(nnz > 0 ? nnz : 1);
  if (std::fread(off.data(), 4, rows + 1, f) != (size_t)rows + 1) return 1;
  if (std::fread(idx.data(), 4, nnz, f) != (size_t)nnz) return 1;
  if (std::fread(val.data(), 4, nnz, f) != (size_t)nnz) return 1;
  if (std::fread(&n, 8, 1, f) != 1) return 1;
  std::vector<float> x(n > 0 ? n : 1);
  if (std::fread(x.data(), 4, n, f) != (size_t)n) return 1;
  std::fclose(f);

  int *d_off, *d_idx, *d_count, *d_ends, *d_mis;
  float *d_val, *d_x, *d_y, *d_y2;
  CHECK(cudaMalloc(&d_off, 4 * (rows + 1)));
  CHECK(cudaMalloc(&d_idx, 4 * idx.size()));
  CHECK(cudaMalloc(&d_val, 4 * val.size()));
  CHECK(cudaMalloc(&d_x, 4 * x.size()));
  CHECK(cudaMalloc(&d_y, 4 * (rows > 0 ? rows : 1)));
  CHECK(cudaMalloc(&d_y2, 4 * (rows > 0 ? rows : 1)));
  CHECK(cudaMalloc(&d_count, 4 * (rows > 0 ? rows : 1)));
  CHECK(cudaMalloc(&d_ends, 4 * (rows > 0 ? rows : 1)));
  CHECK(cudaMalloc(&d_mis, 4));
  CHECK(cudaMemcpy(d_off, off.data(), 4 * (rows + 1), cudaMemcpyHostToDevice));
  CHECK(cudaMemcpy(d_idx, idx.data(), 4 * idx.size(), cudaMemcpyHostToDevice));
  CHECK(cudaMemcpy(d_val, val.data(), 4 * val.size(), cudaMemcpyHostToDevice));
  CHECK(cudaMemcpy(d_x, x.data(), 4 * x.size(), cudaMemcpyHostToDevice));
  CHECK(cudaMemset(d_y, 0, 4 * (rows > 0 ? rows : 1)));
  CHECK(cudaMemset(d_count, 0, 4 * (rows > 0 ? rows : 1)));
  CHECK(cudaMemset(d_ends, 0, 4 * (rows > 0 ? rows : 1)));
  CHECK(cudaMemset(d_mis, 0, 4));
  spmv_ranges<<<37, 128>>>(d_off, d_idx, d_val, d_x, d_y, d_count, d_ends, rows, nnz);
  CHECK(cudaGetLastError());
  spmv_rows<<<23, 128>>>(d_off, d_idx, d_val, d_x, d_y2, rows);
  CHECK(cudaGetLastError());
  check_warp_search<<<64, 256>>>(d_off, rows, nnz, d_mis);
  CHECK(cudaGetLastError());
  CHECK(cudaDeviceSynchronize());

  std::vector<float> y(rows), y2(rows);
  std::vector<int> count(rows), ends(rows);
  int mis = 0;
  CHECK(cudaMemcpy(y.data(), d_y, 4 * rows, cudaMemcpyDeviceToHost));
  CHECK(cudaMemcpy(count.data(), d_count, 4 * rows, cudaMemcpyDeviceToHost));
  CHECK(cudaMemcpy(ends.data(), d_ends, 4 * rows, cudaMemcpyDeviceToHost));
  CHECK(cudaMemcpy(y2.data(), d_y2, 4 * rows, cudaMemcpyDeviceToHost));
  CHECK(cudaMemcpy(&mis, d_mis, 4, cudaMemcpyDeviceToHost));
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 1;
  std::fwrite(y.data(), 4, rows, o);
  std::fwrite(count.data(), 4, rows, o);
  std::fwrite(ends.data(), 4, rows, o);
  std::fwrite(y2.data(), 4, rows, o);
  std::fwrite(&mis, 4, 1, o);
  std::fclose(o);
  return 0;
}
