// edge_loops_schedule.cuh -- the reference's device-side schedule API for
// user kernels: include this header in place of <loops/schedule.hxx> and
// <loops/stride_ranges.hxx> (header-only; no library needed).
//
// A kernel written against the reference's load-balancing API
// (docs/loadbalancing_api.md; include/loops/schedule.hxx:21-46,
// stride_ranges.hxx:16-64, schedule/thread_mapped.hxx:88-166,
// schedule/work_oriented.hxx:86-195, schedule/group_mapped.hxx:80-250,
// schedule/merge_path_flat.hxx:158-436)
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
// per thread of the grid) and strides the group over their nonzeros;
// merge_path_flat cuts the merge of row ends and nonzeros into blocks of
// threads_per_block * items_per_thread items at diagonals k * that size and
// gives each thread items_per_thread consecutive items from diagonal
// threadIdx.x * items_per_thread of its block's tile:
//
//   using setup_t = loops::schedule::setup<loops::schedule::algorithms_t::merge_path_flat,
//                                          threads_per_block, items_per_thread, index_t,
//                                          offset_t, std::size_t, std::size_t>;
//   // host: typename setup_t::meta_t meta(offsets, rows, nnz, stream);
//   __shared__ typename setup_t::storage_t storage;
//   setup_t config(meta, storage, offsets, rows, nnz);
//   auto map = config.init();                    // every thread of the block
//   if (!config.is_valid_accessor(map)) return;
//   for (auto item : config.virtual_idx()) {
//     auto nz = config.atom_idx(item, map);      // clamped to nnz - 1
//     auto row = config.tile_idx(map);
//     if (config.atoms_counting_it[map.y] < storage.tile_end_offset[map.x]) {
//       ... nonzero nz of row `row` ...; map.y++;
//     } else {
//       map.x++;                                 // row `row` ends here
//     }
//   }
//
// Ranges here step forward only.
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

// A (row, nonzero) point of the merge path (the reference's
// coordinate_t, container/coordinate.hxx).
template <typename index_t>
struct coordinate_t {
  index_t x;
  index_t y;
};

// i -> begin + i, as the reference's thrust::counting_iterator is used by
// merge-path loop bodies (it[i], *it).
template <typename T>
struct counting_t {
  T base;
  __host__ __device__ T operator[](long long i) const { return T((long long)base + i); }
  __host__ __device__ T operator*() const { return base; }
};

namespace schedule {

using coord_t = coordinate_t<unsigned int>;

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
class setup;  // every schedule but bucketing is defined below

// ---------------------------------------------------------- merge_path_flat
namespace merge_path {

// The merge-path point of diagonal `diag` of the merge of list a (row ends,
// a_len of them) with the counting list b0, b0 + 1, ... (b_len nonzeros):
// x = the first index in [max(diag - b_len, 0), min(diag, a_len)) where
// a[x] <= b0 + diag - x - 1 fails (the start of the interval when it is
// empty or inverted), point (min(x, a_len), diag - x).  This is the
// reference's search::_binary_search (util/search.hxx:34-60); the failing
// index is unique, so this bisection finds the same point.
template <typename A>
__device__ __forceinline__ coord_t point(long long diag, const A& a, long long a_len,
                                         long long b0, long long b_len) {
  long long lo = diag - b_len > 0 ? diag - b_len : 0;
  long long hi = diag < a_len ? diag : a_len;
  while (lo < hi) {
    const long long mid = lo + ((hi - lo) >> 1);
    if ((long long)a[mid] <= b0 + diag - mid - 1)
      lo = mid + 1;
    else
      hi = mid;
  }
  return coord_t{(unsigned int)(lo < a_len ? lo : a_len), (unsigned int)(diag - lo)};
}

// The reference's preprocess object (schedule/merge_path_flat.hxx:158-230),
// passed to the kernel by value.  The reference may compute every block's
// start point in a separate launch, but its copy constructor leaves the
// kernel's copy without them, so its kernels always search themselves.
// Here nothing is computed or allocated; a caller that has the points
// (el_merge_path_partition writes them: 2 x (tiles + 1) unsigned int) may
// pass them as `tile_coords`, and the blocks then read their start and end
// points from there.
template <std::size_t THREADS_PER_BLOCK, std::size_t ITEMS_PER_THREAD, typename tiles_type,
          typename atoms_type, typename tile_size_type, typename atom_size_type>
class preprocess_t {
 public:
  using tiles_t = tiles_type;
  using atoms_t = atoms_type;
  using tiles_iterator_t = tiles_t*;
  using tile_size_t = tile_size_type;
  using atom_size_t = atom_size_type;

  __host__ preprocess_t(tiles_iterator_t, tile_size_t, atom_size_t, cudaStream_t = 0,
                        coord_t* tile_coords = nullptr)
      : coords_(tile_coords) {}
  __host__ __device__ coord_t* data() const { return coords_; }

 private:
  coord_t* coords_;
};

}  // namespace merge_path

template <std::size_t THREADS_PER_BLOCK, std::size_t ITEMS_PER_THREAD, typename tiles_type,
          typename atoms_type, typename tile_size_type, typename atom_size_type>
class setup<algorithms_t::merge_path_flat, THREADS_PER_BLOCK, ITEMS_PER_THREAD, tiles_type,
            atoms_type, tile_size_type, atom_size_type> {
 public:
  using tiles_t = tiles_type;
  using atoms_t = atoms_type;
  using tiles_iterator_t = tiles_t*;
  using atoms_iterator_t = atoms_t*;
  using tile_size_t = tile_size_type;
  using atom_size_t = atom_size_type;
  using meta_t = merge_path::preprocess_t<THREADS_PER_BLOCK, ITEMS_PER_THREAD, tiles_type,
                                          atoms_type, tile_size_type, atom_size_type>;

  enum : unsigned int {
    threads_per_block = THREADS_PER_BLOCK,
    items_per_thread = ITEMS_PER_THREAD,
    items_per_tile = THREADS_PER_BLOCK * ITEMS_PER_THREAD,
  };

  // Shared state of one block (declare it __shared__ in the kernel): the
  // block's start and end points, and the ends of the rows its tile touches
  // (entry i = end of row start.x + i, the last row's end past the tile) --
  // the loop body compares nonzero indices with them.
  struct storage_t {
    coord_t tile_coords[2];
    tiles_t tile_end_offset[items_per_thread + items_per_tile + 1];
  };

  storage_t& buffer;
  meta_t& meta;
  counting_t<atoms_t> atoms_counting_it;  // tile-local nonzero -> nonzero index
  counting_t<tiles_t> tiles_counting_it;  // tile-local row -> row index

  __device__ __forceinline__ setup(meta_t& _meta, storage_t& _buffer, tiles_iterator_t tiles,
                                   tile_size_t num_tiles, atom_size_t num_atoms)
      : buffer(_buffer),
        meta(_meta),
        atoms_counting_it{atoms_t(0)},
        tiles_counting_it{tiles_t(0)},
        tiles_(tiles),
        num_tiles_(num_tiles),
        num_atoms_(num_atoms),
        num_merge_tiles_(((std::size_t)num_tiles + (std::size_t)num_atoms + items_per_tile - 1) /
                         items_per_tile),
        tile_num_tiles_(0),
        tile_num_atoms_(0) {}

  // Every thread of the block calls this.  Block b (b = blockIdx.x *
  // gridDim.y + blockIdx.y) owns diagonals [b T, (b + 1) T), T =
  // items_per_tile; the thread's point is the tile-local merge-path point of
  // diagonal threadIdx.x * items_per_thread.  Blocks past the last tile get
  // an invalid point (both coordinates all ones).
  __device__ __forceinline__ coord_t init() {
    const std::size_t b = (std::size_t)blockIdx.x * gridDim.y + blockIdx.y;
    if (b >= num_merge_tiles_) return coord_t{~0u, ~0u};
    const long long rows = (long long)num_tiles_, nnz = (long long)num_atoms_;
    if (threadIdx.x < 2) {
      const coord_t* pre = meta.data();
      buffer.tile_coords[threadIdx.x] =
          pre ? pre[b + threadIdx.x]
              : merge_path::point((long long)(b + threadIdx.x) * items_per_tile, tiles_ + 1,
                                  rows, 0, nnz);
    }
    __syncthreads();
    const coord_t st = buffer.tile_coords[0], en = buffer.tile_coords[1];
    tile_num_tiles_ = tile_size_t(en.x - st.x);
    tile_num_atoms_ = atom_size_t(en.y - st.y);
    const long long last = rows - 1;
    for (long long i = threadIdx.x; i < (long long)tile_num_tiles_ + items_per_thread;
         i += threads_per_block) {
      const long long r = (long long)st.x + i < last ? (long long)st.x + i : last;
      buffer.tile_end_offset[i] = tiles_[r + 1];
    }
    atoms_counting_it = counting_t<atoms_t>{atoms_t(st.y)};
    tiles_counting_it = counting_t<tiles_t>{tiles_t(st.x)};
    __syncthreads();
    const coord_t mine = merge_path::point((long long)threadIdx.x * items_per_thread,
                                           buffer.tile_end_offset, (long long)tile_num_tiles_,
                                           (long long)st.y, (long long)tile_num_atoms_);
    __syncthreads();  // the tile state is read-only from here on
    return mine;
  }

  __device__ __forceinline__ bool is_valid_accessor(coord_t& c) const {
    return c.x != ~0u && c.y != ~0u;
  }
  // the thread's items 0 .. items_per_thread - 1
  __device__ __forceinline__ step_range_t<int> virtual_idx() const {
    return custom_stride_range(int(0), int(items_per_thread), int(1));
  }
  // The nonzero index at the point (not advanced), clamped to the last
  // nonzero as the reference clamps it (merge_path_flat.hxx:408-410), so an
  // item that is a row end still reads a valid nonzero.  With no nonzeros
  // at all this is -1, as in the reference: such a matrix has no item to
  // read.
  __device__ __forceinline__ atoms_t atom_idx(int, coord_t& c) const {
    const long long nz = (long long)atoms_counting_it[c.y];
    const long long last = (long long)num_atoms_ - 1;
    return atoms_t(nz < last ? nz : last);
  }
  // the row index at the point (not advanced)
  __device__ __forceinline__ tiles_t tile_idx(coord_t& c) const { return tiles_counting_it[c.x]; }
  // rows ending in, and nonzeros of, this block's tile
  __device__ __forceinline__ tile_size_t num_tiles() const { return tile_num_tiles_; }
  __device__ __forceinline__ atom_size_t num_atoms() const { return tile_num_atoms_; }

 private:
  tiles_iterator_t tiles_;
  tile_size_t num_tiles_;
  atom_size_t num_atoms_;
  std::size_t num_merge_tiles_;
  tile_size_t tile_num_tiles_;
  atom_size_t tile_num_atoms_;
};

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
