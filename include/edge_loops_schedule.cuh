// edge_loops_schedule.cuh -- the reference's device-side schedule API for
// user kernels: include this header in place of <loops/schedule.hxx> and
// <loops/stride_ranges.hxx> (header-only; no library needed).
//
// A kernel written against the reference's load-balancing API
// (docs/loadbalancing_api.md; include/loops/schedule.hxx:21-46,
// stride_ranges.hxx:16-64, schedule/thread_mapped.hxx:88-166,
// schedule/work_oriented.hxx:86-195, schedule/group_mapped.hxx:80-250)
// compiles against this header unchanged (it also replaces
// <loops/util/math.hxx> and <loops/util/launch.hxx>: math::ceil_div,
// launch::non_cooperative, launch::cooperative):
//
//   for (auto i : loops::grid_stride_range(0, n)) ...            // ranges
//
//   using setup_t = loops::schedule::setup<loops::schedule::algorithms_t::thread_mapped,
//                                          1, 1, offset_t, index_t>;
//   setup_t config(offsets, rows, nnz);
//   for (auto row : config.tiles())
//     for (auto nz : config.atoms(row)) ...
//
//   using setup_t = loops::schedule::setup<loops::schedule::algorithms_t::work_oriented,
//                                          threads_per_block, 1, offset_t, index_t>;
//   setup_t config(offsets, rows, nnz);
//   auto map = config.init();
//   for (auto row : config.tiles(map)) for (auto nz : config.atoms(row, map)) ...
//   for (auto row : config.remainder_tiles(map))
//     for (auto nz : config.remainder_atoms(map)) ...
//
//   using setup_t = loops::schedule::block_mapped<threads_per_block, index_t, offset_t>;
//   __shared__ typename setup_t::storage_t storage;          // or warp_mapped
//   setup_t config(storage, offsets, rows, nnz);
//   auto p = config.partition();
//   for (auto v_atom : config.atom_accessor(p)) {
//     auto v_tile = config.tile_accessor(v_atom, p);
//     if (!config.is_valid_accessor(v_tile, p)) continue;
//     auto row = config.tile_id(v_tile, p);
//     auto nz = config.atom_id(v_atom, row, v_tile, p);
//     ...
//   }
//
// Tiles are rows and atoms nonzeros; `tiles` is the row-offsets array
// (rows + 1 entries).  The splits are the reference's: thread_mapped gives
// each thread of the grid rows tid, tid + grid size, ...; work_oriented
// gives thread t the merge-path items [t w, (t + 1) w) of rows + nnz items,
// w = ceil((rows + nnz) / (gridDim.x * threads_per_block)), complete rows
// first, then the part of the row still open at its end; group_mapped gives
// each group of threads_per_tile threads the rows of its threads (one row
// per thread of the grid) and strides the group over their nonzeros.  The
// merge_path_flat setup is not offered: its loop body reads the setup's
// shared-memory tile state directly; edge_loops_device.cuh has the
// merge-path split points and range walk for such kernels.  Ranges here
// step forward only.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace loops {

// [begin, end) walked with a positive step.  A begin at or past the end
// gives an empty range.
template <typename T>
class stepped_range {
 public:
  class iterator {
   public:
    __host__ __device__ iterator(T cur, T step, T end) : cur_(cur), step_(step), end_(end) {}
    __host__ __device__ T operator*() const { return cur_; }
    __host__ __device__ iterator& operator++() {
      cur_ = (end_ - cur_ > step_) ? T(cur_ + step_) : end_;  // never steps past the end
      return *this;
    }
    __host__ __device__ bool operator==(const iterator& o) const { return cur_ == o.cur_; }
    __host__ __device__ bool operator!=(const iterator& o) const { return cur_ != o.cur_; }

   private:
    T cur_, step_, end_;
  };
  __host__ __device__ stepped_range(T begin, T end, T step)
      : begin_(begin < end ? begin : end), end_(end), step_(step > T(0) ? step : T(1)) {}
  __host__ __device__ iterator begin() const { return iterator(begin_, step_, end_); }
  __host__ __device__ iterator end() const { return iterator(end_, step_, end_); }

 private:
  T begin_, end_, step_;
};

// [begin, end) with step 1; step(s) gives the same range with step s.
template <typename T>
class unit_range {
 public:
  class iterator {
   public:
    __host__ __device__ explicit iterator(T cur) : cur_(cur) {}
    __host__ __device__ T operator*() const { return cur_; }
    __host__ __device__ iterator& operator++() {
      ++cur_;
      return *this;
    }
    __host__ __device__ bool operator==(const iterator& o) const { return cur_ == o.cur_; }
    __host__ __device__ bool operator!=(const iterator& o) const { return cur_ != o.cur_; }

   private:
    T cur_;
  };
  __host__ __device__ unit_range(T begin, T end) : begin_(begin < end ? begin : end), end_(end) {}
  __host__ __device__ iterator begin() const { return iterator(begin_); }
  __host__ __device__ iterator end() const { return iterator(end_); }
  __host__ __device__ stepped_range<T> step(T s) const { return stepped_range<T>(begin_, end_, s); }

 private:
  T begin_, end_;
};

template <typename T>
using step_range_t = stepped_range<T>;

template <typename T>
__host__ __device__ __forceinline__ unit_range<T> range(T begin, T end) {
  return unit_range<T>(begin, end);
}

// This thread's items of [begin, end) when the grid's threads take every
// (grid size)-th item.
template <typename T>
__device__ __forceinline__ step_range_t<T> grid_stride_range(T begin, T end) {
  const T tid = T((unsigned long long)blockDim.x * blockIdx.x + threadIdx.x);
  const T threads = T((unsigned long long)gridDim.x * blockDim.x);
  return stepped_range<T>(T(begin + tid), end, threads);
}

// [begin, end) stepped by the block size (the caller adds its own offset).
template <typename T>
__device__ __forceinline__ step_range_t<T> block_stride_range(T begin, T end) {
  return stepped_range<T>(begin, end, T(blockDim.x));
}

template <typename T>
__device__ __forceinline__ step_range_t<T> custom_stride_range(T begin, T end, T stride) {
  return stepped_range<T>(begin, end, stride);
}

// ---- helpers the reference's kernels and launchers use
// (util/math.hxx:26-31, util/launch.hxx:40-74)
namespace math {
// n / d rounded up
template <class numerator_t, class denominator_t>
__host__ __device__ __forceinline__ constexpr numerator_t ceil_div(numerator_t const& n,
                                                                   denominator_t const& d) {
  return static_cast<numerator_t>(n / d + (n % d != 0 ? 1 : 0));
}
}  // namespace math

namespace launch {
// kernel<<<blocks, threads, 0, stream>>>(args...)
template <typename func_t, typename... args_t>
void non_cooperative(cudaStream_t stream, const func_t& kernel, dim3 number_of_blocks,
                     dim3 threads_per_block, args_t&&... args) {
  kernel<<<number_of_blocks, threads_per_block, 0, stream>>>(static_cast<args_t&&>(args)...);
}
// the same as a cooperative launch (every block resident at once; the
// caller sizes the grid to fit)
template <typename func_t, typename... args_t>
cudaError_t cooperative(cudaStream_t stream, const func_t& kernel, std::size_t number_of_blocks,
                        std::size_t threads_per_block, args_t&&... args) {
  void* arg_addresses[sizeof...(args_t) > 0 ? sizeof...(args_t) : 1] = {
      const_cast<void*>(static_cast<const void*>(&args))...};
  return cudaLaunchCooperativeKernel((const void*)kernel, dim3((unsigned)number_of_blocks),
                                     dim3((unsigned)threads_per_block), arg_addresses, 0, stream);
}
}  // namespace launch

namespace schedule {

enum algorithms_t {
  merge_path_flat,
  work_oriented,
  thread_mapped,
  group_mapped,
  bucketing,
};

template <algorithms_t scheme, std::size_t threads_per_block, std::size_t threads_per_tile,
          typename tiles_t, typename atoms_t, typename tile_size_t = std::size_t,
          typename atom_size_t = std::size_t>
class setup;  // thread_mapped, work_oriented and group_mapped are defined below

// ---------------------------------------------------------- thread_mapped
template <typename tiles_type, typename atoms_type, typename tile_size_type,
          typename atom_size_type>
class setup<algorithms_t::thread_mapped, 1, 1, tiles_type, atoms_type, tile_size_type,
            atom_size_type> {
 public:
  using tiles_t = tiles_type;
  using atoms_t = atoms_type;
  using tiles_iterator_t = tiles_t*;
  using tile_size_t = tile_size_type;
  using atom_size_t = atom_size_type;

  __host__ __device__ setup() : tiles_(nullptr), num_tiles_(0), num_atoms_(0) {}
  __host__ __device__ setup(tiles_iterator_t tiles, tile_size_t num_tiles, atom_size_t num_atoms)
      : tiles_(tiles), num_tiles_(num_tiles), num_atoms_(num_atoms) {}

  // this thread's rows: tid, tid + grid size, ...
  __device__ step_range_t<tile_size_t> tiles() const {
    return grid_stride_range(tile_size_t(0), num_tiles_);
  }
  // the nonzeros of row `tile`
  __device__ unit_range<tiles_t> atoms(const tile_size_t& tile) const {
    return range(tiles_[tile], tiles_[tile + 1]);
  }
  // the nonzeros of row `tile` from count_entries(tile) on
  template <typename first_t>
  __device__ unit_range<tiles_t> atoms(const tile_size_t& tile, first_t count_entries) const {
    return range(tiles_t(count_entries(tile)), tiles_[tile + 1]);
  }
  __host__ __device__ tile_size_t size() const { return num_tiles_; }

 private:
  tiles_iterator_t tiles_;
  tile_size_t num_tiles_;
  atom_size_t num_atoms_;
};

// ---------------------------------------------------------- work_oriented
template <typename T>
struct pair_t {
  T first, second;
};

template <std::size_t THREADS_PER_BLOCK, std::size_t ITEMS_PER_THREAD, typename tiles_type,
          typename atoms_type, typename tile_size_type, typename atom_size_type>
class setup<algorithms_t::work_oriented, THREADS_PER_BLOCK, ITEMS_PER_THREAD, tiles_type,
            atoms_type, tile_size_type, atom_size_type> {
 public:
  using tiles_t = tiles_type;
  using atoms_t = atoms_type;
  using tiles_iterator_t = tiles_t*;
  using tile_size_t = tile_size_type;
  using atom_size_t = atom_size_type;
  // (start, end) merge-path points of this thread's share, each (row, nonzero)
  using map_t = pair_t<pair_t<atom_size_t>>;

  enum : unsigned int {
    threads_per_block = THREADS_PER_BLOCK,
    items_per_thread = ITEMS_PER_THREAD,
    items_per_tile = THREADS_PER_BLOCK * ITEMS_PER_THREAD,
  };

  __device__ __forceinline__ setup(tiles_iterator_t tiles, tile_size_t num_tiles,
                                   atom_size_t num_atoms)
      : tiles_(tiles),
        num_tiles_(num_tiles),
        num_atoms_(num_atoms),
        total_work_((std::size_t)num_tiles + (std::size_t)num_atoms),
        num_threads_((std::size_t)gridDim.x * THREADS_PER_BLOCK),
        work_per_thread_((total_work_ + num_threads_ - 1) / num_threads_) {}

  // this thread's share: the points of diagonals t w and (t + 1) w
  __device__ __forceinline__ map_t init() const {
    const std::size_t tid = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x;
    std::size_t upper = work_per_thread_ * tid;
    if (upper > total_work_) upper = total_work_;
    std::size_t lower = upper + work_per_thread_;
    if (lower > total_work_) lower = total_work_;
    map_t m;
    m.first = point(upper);
    m.second = point(lower);
    return m;
  }
  // rows that end inside the share
  template <typename map_type>
  __device__ __forceinline__ step_range_t<tiles_t> tiles(map_type& m) const {
    return custom_stride_range(tiles_t(m.first.first), tiles_t(m.second.first), tiles_t(1));
  }
  // the share's nonzeros of row t (called for the rows of tiles(m) in order;
  // moves the share's start past them)
  template <typename map_type>
  __device__ __forceinline__ step_range_t<atoms_t> atoms(tiles_t t, map_type& m) const {
    const atoms_t b = atoms_t(m.first.second);
    const atoms_t e = atoms_t(tiles_[t + 1]);
    m.first.second = e;
    return custom_stride_range(b, e, atoms_t(1));
  }
  // the row still open at the share's end (the row after the last one when
  // the share ends with a row end; its atom range is then empty)
  template <typename map_type>
  __device__ __forceinline__ step_range_t<tiles_t> remainder_tiles(map_type& m) const {
    return custom_stride_range(tiles_t(m.second.first), tiles_t(m.second.first + 1), tiles_t(1));
  }
  template <typename map_type>
  __device__ __forceinline__ step_range_t<atoms_t> remainder_atoms(map_type& m) const {
    return custom_stride_range(atoms_t(m.first.second), atoms_t(m.second.second), atoms_t(1));
  }

 private:
  // The merge-path point of diagonal d: the first row r in
  // [max(0, d - nnz), min(d, rows)) whose end offsets[r + 1] is above
  // d - r - 1 (the reference's search::_binary_search), and d - r nonzeros.
  __device__ __forceinline__ pair_t<atom_size_t> point(std::size_t d) const {
    std::size_t lo = d > (std::size_t)num_atoms_ ? d - (std::size_t)num_atoms_ : 0;
    std::size_t hi = d < (std::size_t)num_tiles_ ? d : (std::size_t)num_tiles_;
    while (lo < hi) {
      const std::size_t mid = lo + (hi - lo) / 2;
      if ((std::size_t)tiles_[mid + 1] <= d - mid - 1)
        lo = mid + 1;
      else
        hi = mid;
    }
    return pair_t<atom_size_t>{atom_size_t(lo), atom_size_t(d - lo)};
  }

  tiles_iterator_t tiles_;
  tile_size_t num_tiles_;
  atom_size_t num_atoms_;
  std::size_t total_work_, num_threads_, work_per_thread_;
};

// ----------------------------------------------------------- group_mapped
// A group of TPT consecutive threads of a block (the reference's
// cooperative-groups tiled partition): rank in the group, group index in the
// block, group size, and a barrier over the group.
template <std::size_t TPB, std::size_t TPT>
struct thread_group_t {
  static_assert(TPT <= 32 || TPT == TPB,
                "group_mapped groups: up to a warp (a power of two) or the whole block");
  static_assert(TPT == TPB || (32 % TPT == 0), "a group within a warp divides 32");
  __device__ unsigned thread_rank() const { return threadIdx.x % TPT; }
  __device__ unsigned meta_group_rank() const { return threadIdx.x / TPT; }
  __device__ unsigned size() const { return (unsigned)TPT; }
  __device__ void sync() const {
    if (TPT == TPB && TPB > 32)
      __syncthreads();
    else
      __syncwarp();  // the whole warp takes part in every group call
  }
};

template <std::size_t THREADS_PER_BLOCK, std::size_t THREADS_PER_TILE, typename tiles_type,
          typename atoms_type, typename tile_size_type, typename atom_size_type>
class setup<algorithms_t::group_mapped, THREADS_PER_BLOCK, THREADS_PER_TILE, tiles_type,
            atoms_type, tile_size_type, atom_size_type> {
 public:
  using tiles_t = tiles_type;
  using atoms_t = atoms_type;
  using tiles_iterator_t = tiles_t*;
  using tile_size_t = tile_size_type;
  using atom_size_t = atom_size_type;
  using partition_t = thread_group_t<THREADS_PER_BLOCK, THREADS_PER_TILE>;

  enum : unsigned int {
    threads_per_block = THREADS_PER_BLOCK,
    threads_per_tile = THREADS_PER_TILE,
    tiles_per_block = THREADS_PER_BLOCK / THREADS_PER_TILE,
  };
  static_assert(THREADS_PER_BLOCK % 32 == 0, "blocks of whole warps");

  // Shared scratch of one block (declare it __shared__ in the kernel).
  struct __align__(16) storage_t {
    atoms_t tile_aggregates[tiles_per_block];      // nonzeros of each group's rows
    atoms_t atoms_offsets[THREADS_PER_BLOCK];      // exclusive scan of row lengths per group
    tiles_t tiles_indices[THREADS_PER_BLOCK];      // the row of each thread (-1: none)
    atoms_t warp_totals[THREADS_PER_BLOCK / 32];   // block-wide scan scratch
  };

  storage_t& buffer;

  __device__ __forceinline__ setup(storage_t& storage, tiles_iterator_t tiles,
                                   tile_size_t num_tiles, atom_size_t num_atoms)
      : buffer(storage), tiles_(tiles), num_tiles_(num_tiles), num_atoms_(num_atoms) {}

  // Every thread of the block calls this first: thread i of the grid owns
  // row i (if any).
  __device__ __forceinline__ partition_t partition() {
    partition_t p;
    const unsigned long long gid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    buffer.tiles_indices[slot(p)] =
        gid < (unsigned long long)num_tiles_ ? tiles_t(gid) : tiles_t(-1);
    return p;
  }

  // The group's nonzeros (0 .. sum of its rows' lengths), strided over its
  // threads; every thread of the block calls it.
  __device__ step_range_t<atoms_t> atom_accessor(partition_t& p) {
    const unsigned long long gid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    atoms_t len = 0;
    if (gid < (unsigned long long)num_tiles_) len = atoms_t(tiles_[gid + 1] - tiles_[gid]);
    atoms_t total;
    const atoms_t excl = exclusive_scan(p, len, total);
    buffer.atoms_offsets[slot(p)] = excl;
    if (p.thread_rank() == 0) buffer.tile_aggregates[p.meta_group_rank()] = total;
    p.sync();
    return custom_stride_range(atoms_t(p.thread_rank()),
                               atoms_t(buffer.tile_aggregates[p.meta_group_rank()]),
                               atoms_t(p.size()));
  }

  // The group-local row (0 .. rows of the group) that holds the group's
  // nonzero v_atom: the last row whose scanned start is at or below it.
  __device__ __forceinline__ tiles_t tile_accessor(atoms_t& v_atom, partition_t& p) {
    const atoms_t* st = buffer.atoms_offsets + p.meta_group_rank() * p.size();
    int lo = 0, hi = length(p);  // upper bound of v_atom in st[0, length)
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (st[mid] <= v_atom)
        lo = mid + 1;
      else
        hi = mid;
    }
    return tiles_t(lo - 1);
  }
  __device__ __forceinline__ bool is_valid_accessor(tiles_t& v_tile, partition_t& p) {
    const long long t = (long long)v_tile;
    return t >= 0 && t < (long long)length(p);
  }
  // the global row of group-local row v_tile
  __device__ __forceinline__ tiles_t tile_id(tiles_t& v_tile, partition_t& p) {
    return buffer.tiles_indices[p.meta_group_rank() * p.size() + v_tile];
  }
  // the nonzero index of the group's nonzero v_atom, in row `row`
  __device__ __forceinline__ atoms_t atom_id(atoms_t& v_atom, tiles_t& row, tiles_t& v_tile,
                                             partition_t& p) {
    const atoms_t* st = buffer.atoms_offsets + p.meta_group_rank() * p.size();
    return atoms_t(tiles_[row]) + v_atom - st[v_tile];
  }

 private:
  __device__ static unsigned slot(const partition_t& p) {
    return p.meta_group_rank() * p.size() + p.thread_rank();
  }
  // rows owned by the group: its threads' indices below num_tiles
  __device__ int length(const partition_t& p) const {
    const long long first = (long long)blockIdx.x * blockDim.x +
                            (long long)p.meta_group_rank() * p.size();
    long long n = (long long)num_tiles_ - first;
    if (n > (long long)p.size()) n = p.size();
    return n > 0 ? (int)n : 0;
  }
  // exclusive scan of v over the group (in thread-rank order) and its total
  __device__ atoms_t exclusive_scan(partition_t& p, atoms_t v, atoms_t& total) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned width = THREADS_PER_TILE < 32 ? (unsigned)THREADS_PER_TILE : 32u;
    atoms_t inc = v;  // inclusive scan within min(group, warp)
    for (unsigned d = 1; d < width; d <<= 1) {
      const atoms_t o = __shfl_up_sync(0xffffffffu, inc, d, width);
      if ((lane % width) >= d) inc += o;
    }
    if (THREADS_PER_TILE <= 32) {
      total = __shfl_sync(0xffffffffu, inc, (int)(width - 1), width);
      return inc - v;
    }
    // whole block: add the totals of the earlier warps
    const unsigned warp = threadIdx.x >> 5;
    if (lane == 31) buffer.warp_totals[warp] = inc;
    __syncthreads();
    atoms_t before = 0, all = 0;
    for (unsigned w = 0; w < THREADS_PER_BLOCK / 32; ++w) {
      const atoms_t t = buffer.warp_totals[w];
      if (w < warp) before += t;
      all += t;
    }
    total = all;
    __syncthreads();  // warp_totals may be reused by the next call
    return before + inc - v;
  }

  tiles_iterator_t tiles_;
  tile_size_t num_tiles_;
  atom_size_t num_atoms_;
};

template <std::size_t threads_per_block, typename tiles_t, typename atoms_t>
using warp_mapped = setup<algorithms_t::group_mapped, threads_per_block, 32, tiles_t, atoms_t>;

template <std::size_t threads_per_block, typename tiles_t, typename atoms_t>
using block_mapped =
    setup<algorithms_t::group_mapped, threads_per_block, threads_per_block, tiles_t, atoms_t>;

}  // namespace schedule
}  // namespace loops
