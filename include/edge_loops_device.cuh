// edge_loops_device.cuh -- device-side load-balanced loops over a CSR
// matrix, for user kernels (header-only; no library needed).
//
// This is the counterpart of the reference's schedule API
// (include/loops/schedule.hxx, schedule/merge_path_flat.hxx:108-436,
// schedule/thread_mapped.hxx:88-166; docs/loadbalancing_api.md): a user
// kernel asks for its share of the work and runs its own loop body on each
// (row, nonzero) pair, the split being independent of the body.
//
//   * merge_path_search   -- the split point of a merge-path diagonal, with
//     the reference's search::_binary_search semantics (util/search.hxx:
//     34-60): the rows closed before the diagonal and its nonzero index;
//   * warp_merge_path_search -- the same point found by a whole warp (33
//     candidates per round, so 2^20 rows take 4 rounds);
//   * merge_path_range    -- the merge path of rows + nnz items cut into
//     `parts` equal ranges: the begin and end points of one part;
//   * for_each_in_range   -- a thread walks one range in merge order and
//     calls on_nonzero(row, nz) for every nonzero and on_row_end(row) for
//     every row that ends inside the range (after that row's nonzeros);
//   * for_each_row        -- the thread-mapped loop: rows strided over the
//     grid, on_nonzero(row, nz) then on_row_end(row) per row;
//   * edge_tiles / for_each_tile_quark -- the tiles of an edge partition
//     (quarks grouped into atoms and tiles, edge_loops.h) walked a tile per
//     thread, the reference's schedule_edge thread_mapped setup.
//
// A row that crosses ranges gets on_nonzero calls from several threads and
// on_row_end from the thread whose range contains its end; combining the
// partial results (atomics, or a carry exchange) is the body's business.
// Offsets are int32 with offsets[0] == 0 and offsets[rows] == nnz, as in the
// reference; rows + nnz must be below 2^31.
#pragma once

#include <cuda_runtime.h>

namespace edge_loops {
namespace device {

// A point of the merge path: `row` rows are closed, `nz` nonzeros consumed.
struct coord {
  int row;
  int nz;
};

// Lower bound over rows i in [max(0, d - nnz), min(d, rows)) of
// offsets[i + 1] > d - i - 1: the point where diagonal d crosses the merge
// path of the row ends (offsets + 1) and the nonzero indices.
__device__ __forceinline__ coord merge_path_search(const int* offsets, int rows, int nnz,
                                                   long long d) {
  long long lo = d - nnz > 0 ? d - nnz : 0;
  long long hi = d < rows ? d : rows;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if ((long long)offsets[mid + 1] <= d - mid - 1)
      lo = mid + 1;
    else
      hi = mid;
  }
  return coord{(int)lo, (int)(d - lo)};
}

// merge_path_search by a whole warp; every lane of the warp must call it
// with the same arguments, and every lane gets the result.
__device__ __forceinline__ coord warp_merge_path_search(const int* offsets, int rows, int nnz,
                                                        long long d) {
  const int lane = threadIdx.x & 31;
  long long lo = d - nnz > 0 ? d - nnz : 0;
  long long hi = d < rows ? d : rows;
  while (hi - lo > 32) {
    const long long span = hi - lo;
    const long long p = lo + ((long long)(lane + 1) * span) / 33;
    const bool t = (long long)offsets[p + 1] <= d - p - 1;
    const int c = __popc(__ballot_sync(0xffffffffu, t));
    const long long plo = __shfl_sync(0xffffffffu, p, c > 0 ? c - 1 : 0);
    const long long phi = __shfl_sync(0xffffffffu, p, c < 32 ? c : 31);
    if (c > 0) lo = plo + 1;
    if (c < 32) hi = phi;
  }
  const long long p = lo + lane;
  const bool t = p < hi && (long long)offsets[p + 1] <= d - p - 1;
  const long long x = lo + __popc(__ballot_sync(0xffffffffu, t));
  return coord{(int)x, (int)(d - x)};
}

// Part `p` of `parts` equal ranges of the rows + nnz merge items (the last
// parts may be shorter): its begin and end points.
__device__ __forceinline__ void merge_path_range(const int* offsets, int rows, int nnz,
                                                 long long parts, long long p, coord& begin,
                                                 coord& end) {
  const long long total = (long long)rows + nnz;
  const long long per = (total + parts - 1) / parts;
  long long d0 = p * per, d1 = d0 + per;
  if (d0 > total) d0 = total;
  if (d1 > total) d1 = total;
  begin = merge_path_search(offsets, rows, nnz, d0);
  end = merge_path_search(offsets, rows, nnz, d1);
}

// Walks the merge path from `begin` to `end`: a nonzero is consumed while
// it lies before the end of the current row, otherwise the row is closed.
template <typename OnNonzero, typename OnRowEnd>
__device__ __forceinline__ void for_each_in_range(const int* offsets, coord begin, coord end,
                                                  OnNonzero on_nonzero, OnRowEnd on_row_end) {
  int row = begin.row, nz = begin.nz;
  while (row < end.row || nz < end.nz) {
    const int row_end = offsets[row + 1];
    if (row < end.row && nz >= row_end) {
      on_row_end(row);
      ++row;
    } else {
      on_nonzero(row, nz);
      ++nz;
    }
  }
}

// The thread-mapped loop: each thread of the grid takes rows tid,
// tid + grid size, ... and visits their nonzeros in order.
template <typename OnNonzero, typename OnRowEnd>
__device__ __forceinline__ void for_each_row(const int* offsets, int rows, OnNonzero on_nonzero,
                                             OnRowEnd on_row_end) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += stride) {
    const int b = offsets[r], e = offsets[r + 1];
    for (int nz = b; nz < e; ++nz) on_nonzero((int)r, nz);
    on_row_end((int)r);
  }
}

// ---- edge partitions ----------------------------------------------------
// The tiles of an edge partition (el_edge_partition of edge_loops.h, built
// by el_edge_partition_coordinate / _position), for user kernels: the
// reference's schedule_edge::setup<thread_mapped>
// (schedule_edge/thread_mapped.hxx:45-117), whose tiles() / atoms(tile) /
// quarks(atom) ranges are index ranges into the partition's arrays here.
struct edge_tiles {
  const int* quarks;      // nnz: COO positions, tile by tile, atom by atom
  const int* atom_begin;  // atoms + 1
  const int* tile_begin;  // tiles + 1
  long long num_tiles;

  __device__ int atoms_begin(long long tile) const { return tile_begin[tile]; }
  __device__ int atoms_end(long long tile) const { return tile_begin[tile + 1]; }
  __device__ int quarks_begin(int atom) const { return atom_begin[atom]; }
  __device__ int quarks_end(int atom) const { return atom_begin[atom + 1]; }
};

// The thread-mapped tile loop: each thread of the grid takes tiles tid,
// tid + grid size, ... and calls on_quark(tile, atom, q) for every quark q
// (a COO position) of every atom of the tile, in partition order.
template <typename OnQuark>
__device__ __forceinline__ void for_each_tile_quark(const edge_tiles& P, OnQuark on_quark) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < P.num_tiles;
       t += stride)
    for (int a = P.atoms_begin(t); a < P.atoms_end(t); ++a)
      for (int i = P.quarks_begin(a); i < P.quarks_end(a); ++i) on_quark(t, a, P.quarks[i]);
}

}  // namespace device
}  // namespace edge_loops
