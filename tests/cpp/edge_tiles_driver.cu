// edge_tiles_driver.cu -- a user kernel written with the edge-partition loop
// of include/edge_loops_device.cuh (for_each_tile_quark), run on a COO and a
// partition read from a file:
//   in : int64 rows, cols, nnz, num_atoms, num_tiles; int32 row[nnz];
//        int32 col[nnz]; float val[nnz]; float x[cols]; int32 quarks[nnz];
//        int32 atom_begin[num_atoms + 1]; int32 tile_begin[num_tiles + 1]
//   out: float y[rows] (atomics, as the reference's edge example);
//        int32 tile[nnz] (the tile that visited each quark);
//        int32 visits[nnz] (how many times each quark was visited)
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

__global__ void spmv_tiles(eld::edge_tiles P, const int* row, const int* col, const float* val,
                           const float* x, float* y, int* tile, int* visits) {
  eld::for_each_tile_quark(P, [&](long long t, int, int q) {
    atomicAdd(y + row[q], val[q] * x[col[q]]);
    tile[q] = (int)t;
    atomicAdd(visits + q, 1);
  });
}

template <typename T>
static T* upload(const std::vector<T>& h) {
  T* d = nullptr;
  CHECK(cudaMalloc(&d, sizeof(T) * (h.empty() ? 1 : h.size())));
  if (!h.empty()) CHECK(cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return d;
}

template <typename T>
static bool read(FILE* f, std::vector<T>& v, long long n) {
  v.resize((size_t)n);
  return n == 0 || std::fread(v.data(), sizeof(T), (size_t)n, f) == (size_t)n;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 1;
  long long h[5];
  if (std::fread(h, 8, 5, f) != 5) return 1;
  const long long rows = h[0], cols = h[1], nnz = h[2], atoms = h[3], tiles = h[4];
  std::vector<int> row, col, quarks, ab, tb;
  std::vector<float> val, x;
  if (!read(f, row, nnz) || !read(f, col, nnz) || !read(f, val, nnz) || !read(f, x, cols) ||
      !read(f, quarks, nnz) || !read(f, ab, atoms + 1) || !read(f, tb, tiles + 1))
    return 1;
  std::fclose(f);
  int *d_row = upload(row), *d_col = upload(col), *d_q = upload(quarks), *d_ab = upload(ab),
      *d_tb = upload(tb);
  float *d_val = upload(val), *d_x = upload(x);
  float* d_y = upload(std::vector<float>((size_t)rows, 0.f));
  int* d_tile = upload(std::vector<int>((size_t)nnz, -1));
  int* d_vis = upload(std::vector<int>((size_t)nnz, 0));
  eld::edge_tiles P{d_q, d_ab, d_tb, tiles};
  spmv_tiles<<<13, 64>>>(P, d_row, d_col, d_val, d_x, d_y, d_tile, d_vis);
  CHECK(cudaGetLastError());
  CHECK(cudaDeviceSynchronize());
  std::vector<float> y((size_t)rows);
  std::vector<int> tile((size_t)nnz), vis((size_t)nnz);
  if (rows) CHECK(cudaMemcpy(y.data(), d_y, 4 * rows, cudaMemcpyDeviceToHost));
  if (nnz) CHECK(cudaMemcpy(tile.data(), d_tile, 4 * nnz, cudaMemcpyDeviceToHost));
  if (nnz) CHECK(cudaMemcpy(vis.data(), d_vis, 4 * nnz, cudaMemcpyDeviceToHost));
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 1;
  std::fwrite(y.data(), 4, y.size(), o);
  std::fwrite(tile.data(), 4, tile.size(), o);
  std::fwrite(vis.data(), 4, vis.size(), o);
  std::fclose(o);
  return 0;
}
