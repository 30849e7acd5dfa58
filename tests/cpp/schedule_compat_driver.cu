// schedule_compat_driver.cu -- user kernels written the way the reference's
// load-balancing API documents them (loops::schedule::setup, ranged loops),
// compiled against include/edge_loops_schedule.cuh instead of the
// reference's headers, run on a CSR read from a file:
//   in : int64 rows, cols, nnz; int32 offsets[rows+1]; int32 indices[nnz];
//        float values[nnz]; int64 n; float x[n]
//   out: float y_thread[rows]  (thread_mapped setup: rows in order, y stored)
//        float y_work[rows]    (work_oriented setup: whole rows stored, the
//                               open row of each share added atomically)
//        float y_warp[rows]    (warp_mapped setup, atomics)
//        float y_block[rows]   (block_mapped setup, atomics)
//        int32 visits[nnz]     (block_mapped: times each nonzero was visited)
//        float z[n]            (2 x + z0 by grid_stride_range, z0 = 1)
//        float y_merge[rows]   (merge_path_flat setup, 128 x 5 items per
//                               block, atomics, as the reference's kernel)
//        uint32 coords[tiles * 128 * 2]  (each thread's tile-local start
//                               point from init(); tiles = ceil((rows +
//                               nnz) / 640); skipped when nnz == 0)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <edge_loops_schedule.cuh>

using namespace loops;

#define CHECK(x)                                                              \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));          \
      std::exit(1);                                                           \
    }                                                                         \
  } while (0)

__global__ void saxpy(int n, float a, const float* x, float* z) {
  for (auto i : grid_stride_range(0, n)) z[i] += a * x[i];
}

template <typename index_t, typename offset_t, typename type_t>
__global__ void spmv_thread_mapped(std::size_t rows, std::size_t cols, std::size_t nnz,
                                   offset_t* offsets, index_t* indices, const type_t* values,
                                   const type_t* x, type_t* y) {
  using setup_t = schedule::setup<schedule::algorithms_t::thread_mapped, 1, 1, index_t,
                                  offset_t, std::size_t, std::size_t>;
  setup_t config(offsets, rows, nnz);
  for (auto row : config.tiles()) {
    type_t sum = 0;
    for (auto nz : config.atoms(row)) sum += values[nz] * x[indices[nz]];
    y[row] = sum;
  }
}

template <std::size_t threads_per_block, typename index_t, typename offset_t, typename type_t>
__global__ void spmv_work_oriented(std::size_t rows, std::size_t cols, std::size_t nnz,
                                   offset_t* offsets, index_t* indices, const type_t* values,
                                   const type_t* x, type_t* y) {
  using setup_t = schedule::setup<schedule::algorithms_t::work_oriented, threads_per_block, 1,
                                  index_t, offset_t, std::size_t, std::size_t>;
  setup_t config(offsets, rows, nnz);
  auto map = config.init();
  type_t sum = 0;
  for (auto row : config.tiles(map)) {
    for (auto nz : config.atoms(row, map)) sum += values[nz] * x[indices[nz]];
    atomicAdd(&y[row], sum);  // a row begun in an earlier share gets two parts
    sum = 0;
  }
  for (auto row : config.remainder_tiles(map)) {
    for (auto nz : config.remainder_atoms(map)) sum += values[nz] * x[indices[nz]];
    if (sum != 0) atomicAdd(&y[row], sum);
  }
}

template <typename setup_t, typename index_t, typename offset_t, typename type_t>
__device__ void group_body(typename setup_t::storage_t& storage, std::size_t rows,
                           std::size_t nnz, offset_t* offsets, index_t* indices,
                           const type_t* values, const type_t* x, type_t* y, int* visits) {
  setup_t config(storage, offsets, rows, nnz);
  auto p = config.partition();
  for (auto virtual_atom : config.atom_accessor(p)) {
    auto virtual_tile = config.tile_accessor(virtual_atom, p);
    if (!(config.is_valid_accessor(virtual_tile, p))) continue;
    auto row = config.tile_id(virtual_tile, p);
    auto nz_idx = config.atom_id(virtual_atom, row, virtual_tile, p);
    atomicAdd(&(y[row]), values[nz_idx] * x[indices[nz_idx]]);
    if (visits) atomicAdd(visits + nz_idx, 1);
  }
}

template <std::size_t threads_per_block, typename index_t, typename offset_t, typename type_t>
__global__ void spmv_warp_mapped(std::size_t rows, std::size_t cols, std::size_t nnz,
                                 offset_t* offsets, index_t* indices, const type_t* values,
                                 const type_t* x, type_t* y) {
  using setup_t = schedule::warp_mapped<threads_per_block, index_t, offset_t>;
  __shared__ typename setup_t::storage_t storage;
  group_body<setup_t>(storage, rows, nnz, offsets, indices, values, x, y, (int*)nullptr);
}

template <std::size_t threads_per_block, typename index_t, typename offset_t, typename type_t>
__global__ void spmv_block_mapped(std::size_t rows, std::size_t cols, std::size_t nnz,
                                  offset_t* offsets, index_t* indices, const type_t* values,
                                  const type_t* x, type_t* y, int* visits) {
  using setup_t = schedule::block_mapped<threads_per_block, index_t, offset_t>;
  __shared__ typename setup_t::storage_t storage;
  group_body<setup_t>(storage, rows, nnz, offsets, indices, values, x, y, visits);
}

template <std::size_t threads_per_block, std::size_t items_per_thread, typename meta_t,
          typename index_t, typename offset_t, typename type_t>
__global__ void spmv_merge_path(meta_t meta, std::size_t rows, std::size_t cols, std::size_t nnz,
                                offset_t* offsets, index_t* indices, const type_t* values,
                                const type_t* x, type_t* y, unsigned* coords) {
  using setup_t = schedule::setup<schedule::algorithms_t::merge_path_flat, threads_per_block,
                                  items_per_thread, index_t, offset_t, std::size_t,
                                  std::size_t>;
  __shared__ typename setup_t::storage_t storage;
  setup_t config(meta, storage, offsets, rows, nnz);
  auto map = config.init();
  if (!config.is_valid_accessor(map)) return;
  const std::size_t t = (std::size_t)blockIdx.x * threads_per_block + threadIdx.x;
  coords[2 * t] = map.x;
  coords[2 * t + 1] = map.y;
  for (auto item : config.virtual_idx()) {
    auto nz = config.atom_idx(item, map);
    auto row = config.tile_idx(map);
    type_t nonzero = values[nz] * x[indices[nz]];
    if (config.atoms_counting_it[map.y] < storage.tile_end_offset[map.x]) {
      atomicAdd(&(y[row]), nonzero);
      map.y++;
    } else {
      map.x++;
    }
  }
}

template <typename T>
static T* upload(const std::vector<T>& h) {
  T* d = nullptr;
  CHECK(cudaMalloc(&d, (h.size() > 0 ? h.size() : 1) * sizeof(T)));
  if (!h.empty()) CHECK(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return d;
}

template <typename T>
static std::vector<T> download(const T* d, size_t n) {
  std::vector<T> h(n);
  if (n) CHECK(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost));
  return h;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  long long hdr[3], n = 0;
  if (std::fread(hdr, sizeof(long long), 3, f) != 3) return 2;
  const long long rows = hdr[0], cols = hdr[1], nnz = hdr[2];
  std::vector<int> off(rows + 1), idx(nnz);
  std::vector<float> val(nnz);
  if (std::fread(off.data(), 4, rows + 1, f) != (size_t)(rows + 1)) return 2;
  if (nnz && std::fread(idx.data(), 4, nnz, f) != (size_t)nnz) return 2;
  if (nnz && std::fread(val.data(), 4, nnz, f) != (size_t)nnz) return 2;
  if (std::fread(&n, sizeof(long long), 1, f) != 1 || n != cols) return 2;
  std::vector<float> x(n);
  if (n && std::fread(x.data(), 4, n, f) != (size_t)n) return 2;
  std::fclose(f);

  int* d_off = upload(off);
  int* d_idx = upload(idx);
  float* d_val = upload(val);
  float* d_x = upload(x);
  const size_t ry = rows > 0 ? (size_t)rows : 1;
  float *d_y1, *d_y2, *d_y3, *d_y4, *d_z;
  int* d_vis;
  CHECK(cudaMalloc(&d_y1, ry * 4));
  CHECK(cudaMalloc(&d_y2, ry * 4));
  CHECK(cudaMalloc(&d_y3, ry * 4));
  CHECK(cudaMalloc(&d_y4, ry * 4));
  CHECK(cudaMalloc(&d_vis, (nnz > 0 ? nnz : 1) * 4));
  CHECK(cudaMalloc(&d_z, (n > 0 ? n : 1) * 4));
  CHECK(cudaMemset(d_y2, 0, ry * 4));
  CHECK(cudaMemset(d_y3, 0, ry * 4));
  CHECK(cudaMemset(d_y4, 0, ry * 4));
  CHECK(cudaMemset(d_vis, 0, (nnz > 0 ? nnz : 1) * 4));
  std::vector<float> ones(n, 1.0f);
  if (n) CHECK(cudaMemcpy(d_z, ones.data(), n * 4, cudaMemcpyHostToDevice));

  constexpr std::size_t tpb = 128;
  const unsigned row_blocks = (unsigned)math::ceil_div((std::size_t)rows, tpb);
  if (rows > 0) {
    // a small grid, so that threads take several rows / a long share each
    spmv_thread_mapped<int, int, float><<<7, tpb>>>(rows, cols, nnz, d_off, d_idx, d_val, d_x,
                                                    d_y1);
    spmv_work_oriented<tpb, int, int, float><<<5, tpb>>>(rows, cols, nnz, d_off, d_idx, d_val,
                                                         d_x, d_y2);
    spmv_warp_mapped<tpb, int, int, float><<<row_blocks, tpb>>>(rows, cols, nnz, d_off, d_idx,
                                                                d_val, d_x, d_y3);
    launch::non_cooperative(nullptr, spmv_block_mapped<tpb, int, int, float>, row_blocks, tpb,
                            (std::size_t)rows, (std::size_t)cols, (std::size_t)nnz, d_off, d_idx,
                            (const float*)d_val, (const float*)d_x, d_y4, d_vis);
  }
  if (n) saxpy<<<3, 64>>>((int)n, 2.0f, d_x, d_z);
  // merge_path_flat: one block per tile of 128 x 5 merge items
  constexpr std::size_t ipt = 5;
  const std::size_t tiles = math::ceil_div((std::size_t)(rows + nnz), tpb * ipt);
  float* d_y5;
  unsigned* d_coords;
  CHECK(cudaMalloc(&d_y5, ry * 4));
  CHECK(cudaMemset(d_y5, 0, ry * 4));
  CHECK(cudaMalloc(&d_coords, (tiles > 0 ? tiles : 1) * tpb * 2 * 4));
  CHECK(cudaMemset(d_coords, 0xff, (tiles > 0 ? tiles : 1) * tpb * 2 * 4));
  if (rows > 0 && nnz > 0) {
    using meta_t = schedule::merge_path::preprocess_t<tpb, ipt, int, int, std::size_t,
                                                      std::size_t>;
    meta_t meta(d_off, (std::size_t)rows, (std::size_t)nnz);
    spmv_merge_path<tpb, ipt, meta_t, int, int, float><<<(unsigned)tiles, tpb>>>(
        meta, rows, cols, nnz, d_off, d_idx, d_val, d_x, d_y5, d_coords);
  }
  CHECK(cudaGetLastError());
  CHECK(cudaDeviceSynchronize());

  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  auto put = [&](const void* p, size_t bytes) { std::fwrite(p, 1, bytes, o); };
  for (float* d : {d_y1, d_y2, d_y3, d_y4}) {
    auto h = download(d, (size_t)rows);
    put(h.data(), h.size() * 4);
  }
  auto vis = download(d_vis, (size_t)nnz);
  put(vis.data(), vis.size() * 4);
  auto z = download(d_z, (size_t)n);
  put(z.data(), z.size() * 4);
  auto y5 = download(d_y5, (size_t)rows);
  put(y5.data(), y5.size() * 4);
  auto co = download(d_coords, nnz > 0 ? tiles * tpb * 2 : 0);
  put(co.data(), co.size() * 4);
  std::fclose(o);
  return 0;
}
