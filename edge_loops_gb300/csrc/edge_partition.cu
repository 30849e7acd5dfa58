// edge_partition.cu -- the edge (nonzero) partitioner and the SpMV over its
// tiles, the reference's util/partitioner.hxx:68-301 and
// schedule_edge/thread_mapped.hxx:45-117 (with the kernel of
// examples/spmv/thread_mapped_edge.cu:16-34), plus the COO helpers it needs
// (coo_t::sort_by_row / sort_by_column, coo.hxx:104-122, and the COO of a
// CSR, coo.hxx:90-97).
//
// The work units are the reference's: a quark is one nonzero (its position
// in the COO), an atom a set of quarks, a tile a set of atoms.
//
//   coordinate space: atom (ax, ay) holds the nonzeros of rows
//     [ax M0, ax M0 + M0) and columns [ay K0, ay K0 + K0), in COO order
//     [partitioner.hxx:81-127]; atoms are numbered row-major over the
//     ceil(rows/M0) x ceil(cols/K0) grid; tile (tx, ty) holds the atoms of
//     atom rows [tx M1, ..) and atom columns [ty K1, ..), tiles row-major,
//     the atoms of a tile in atom order [:129-176];
//   position space: atom i holds quarks [i P, min(i P + P, nnz)), tile t
//     atoms [t T, min(t T + T, atoms)) [:178-226].
//
// Layout (GB300): the partition is three CSR-like arrays instead of the
// reference's pointer-carrying WorkAtom / WorkTile structs -- quarks in tile
// order then atom order, atom_begin (the atoms' quark ranges, in tile order)
// and tile_begin (the tiles' atom ranges) -- so a tile's quarks are one
// contiguous range and a warp reads them coalesced.  The coordinate-space
// order of the atoms is a closed form (the rank below), so the partition is
// one stable radix sort of the quarks by the rank of their atom, one search
// per atom, and closed-form atom coordinates and tile starts.
//
// The reference's prepare_gpu() [:228-258] re-points the device atoms at
// running sums taken in tile order while the device quarks stay in atom
// order, so with M1 > 1 and K1 < the atom columns its device tiles read
// other atoms' quarks; the partition here follows the host-side structure it
// builds [:113-124, :162-173], which is what it intends.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>

#include "el_internal.h"

namespace el {
namespace {

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

int bits_for(long long n) {  // bits to hold the values 0 .. n-1
  int b = 1;
  while (b < 62 && (1LL << b) < n) ++b;
  return b;
}

// The coordinate-space atom and tile grids.
struct Grid {
  long long M0, K0, M1, K1;
  long long nax, nay;  // atoms along rows, columns
  long long ntx, nty;  // tiles along atom rows, atom columns

  // position of atom (ax, ay) in tile order: the atoms of earlier tile rows
  // (M1 full atom rows each), of earlier tiles in this tile row (h atom rows
  // by K1 atom columns each), then row-major inside the tile (h by w)
  __host__ __device__ long long rank(long long ax, long long ay) const {
    const long long tx = ax / M1, ty = ay / K1;
    const long long h = min(M1, nax - tx * M1), w = min(K1, nay - ty * K1);
    return tx * M1 * nay + h * ty * K1 + (ax - tx * M1) * w + (ay - ty * K1);
  }
  __host__ __device__ long long tile_start(long long tx, long long ty) const {
    const long long h = min(M1, nax - tx * M1);
    return tx * M1 * nay + h * ty * K1;
  }
  __host__ __device__ void unrank(long long rk, long long& ax, long long& ay) const {
    const long long tx = rk / (M1 * nay);
    const long long rem = rk - tx * M1 * nay;
    const long long h = min(M1, nax - tx * M1);
    const long long ty = rem / (h * K1);
    const long long rem2 = rem - ty * h * K1;
    const long long w = min(K1, nay - ty * K1);
    ax = tx * M1 + rem2 / w;
    ay = ty * K1 + rem2 % w;
  }
};

__global__ void rank_kernel(const int32_t* __restrict__ ri, const int32_t* __restrict__ ci,
                            long long nnz, long long rows, long long cols, Grid g,
                            unsigned long long* __restrict__ keys, int32_t* __restrict__ pos,
                            unsigned* __restrict__ bad) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = ri[k], c = ci[k];
    unsigned long long key = 0;
    if ((unsigned long long)(unsigned)r >= (unsigned long long)rows ||
        (unsigned long long)(unsigned)c >= (unsigned long long)cols)
      atomicOr(bad, 1u);
    else
      key = (unsigned long long)g.rank(r / g.M0, c / g.K0);
    keys[k] = key;
    pos[k] = (int32_t)k;
  }
}

// atom_begin[a] = the first sorted position whose rank is >= a, a = 0..atoms
__global__ void atom_begin_kernel(const unsigned long long* __restrict__ keys, long long nnz,
                                  long long atoms, int32_t* __restrict__ atom_begin) {
  for (long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x; a <= atoms;
       a += (long long)gridDim.x * blockDim.x) {
    long long lo = 0, hi = nnz;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (keys[mid] < (unsigned long long)a) lo = mid + 1; else hi = mid;
    }
    atom_begin[a] = (int32_t)lo;
  }
}

__global__ void atom_coord_kernel(Grid g, long long atoms, int32_t* __restrict__ ax,
                                  int32_t* __restrict__ ay) {
  for (long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x; a < atoms;
       a += (long long)gridDim.x * blockDim.x) {
    long long x, y;
    g.unrank(a, x, y);
    ax[a] = (int32_t)x;
    ay[a] = (int32_t)y;
  }
}

__global__ void tile_begin_kernel(Grid g, long long tiles, long long atoms,
                                  int32_t* __restrict__ tile_begin) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t <= tiles;
       t += (long long)gridDim.x * blockDim.x)
    tile_begin[t] = (int32_t)(t == tiles ? atoms : g.tile_start(t / g.nty, t % g.nty));
}

// position space: quarks in order, equal atoms and tiles, atom coordinates 0
// (the reference's WorkAtom(quarks, n) sets x_idx = y_idx = 0)
__global__ void position_kernel(long long nnz, long long per_atom, long long atoms,
                                long long per_tile, long long tiles, int32_t* __restrict__ quarks,
                                int32_t* __restrict__ atom_begin, int32_t* __restrict__ ax,
                                int32_t* __restrict__ ay, int32_t* __restrict__ tile_begin) {
  const long long n = max(nnz, atoms + 1);
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    if (k < nnz) quarks[k] = (int32_t)k;
    if (k <= atoms) atom_begin[k] = (int32_t)min(k * per_atom, nnz);
    if (k < atoms) ax[k] = ay[k] = 0;
    if (k <= tiles) tile_begin[k] = (int32_t)min(k * per_tile, atoms);
  }
}

// coo_t::sort_by_row / sort_by_column: keys (major << 31 | minor)
__global__ void coo_keys_kernel(const int32_t* __restrict__ ri, const int32_t* __restrict__ ci,
                                long long nnz, long long rows, long long cols, int by_column,
                                unsigned long long* __restrict__ keys, int32_t* __restrict__ pos,
                                unsigned* __restrict__ bad) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = ri[k], c = ci[k];
    if ((unsigned long long)(unsigned)r >= (unsigned long long)rows ||
        (unsigned long long)(unsigned)c >= (unsigned long long)cols)
      atomicOr(bad, 1u);
    const unsigned hi = by_column ? (unsigned)c : (unsigned)r;
    const unsigned lo = by_column ? (unsigned)r : (unsigned)c;
    keys[k] = ((unsigned long long)hi << 31) | lo;
    pos[k] = (int32_t)k;
  }
}

__global__ void coo_scatter_kernel(const unsigned long long* __restrict__ keys,
                                   const int32_t* __restrict__ pos,
                                   const float* __restrict__ vin, long long nnz, int by_column,
                                   int32_t* __restrict__ ri, int32_t* __restrict__ ci,
                                   float* __restrict__ vout) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (long long)gridDim.x * blockDim.x) {
    const unsigned long long key = keys[k];
    const int32_t hi = (int32_t)(key >> 31), lo = (int32_t)(key & 0x7fffffffull);
    ri[k] = by_column ? lo : hi;
    ci[k] = by_column ? hi : lo;
    vout[k] = vin[pos[k]];
  }
}

// row index of every nonzero: a warp per row, its lanes write the row's run
__global__ void row_indices_kernel(const int32_t* __restrict__ offsets, long long rows,
                                   int32_t* __restrict__ ri) {
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows;
       r += warps) {
    const int b = offsets[r], e = offsets[r + 1];
    for (int k = b + lane; k < e; k += 32) ri[k] = (int32_t)r;
  }
}

}  // namespace
}  // namespace el

namespace el {
namespace {

// y[row] += the products of each tile's quarks, a warp per tile (tiles
// strided over the grid's warps, the reference's thread-mapped tile loop
// with a warp in place of a thread): 32 quarks at a time, coalesced reads
// of the tile's quark range, the products of equal adjacent rows summed in
// registers and added to y once per run.  Quarks, rows and columns outside
// the arrays are skipped and raise EL_FLAG_INDEX_RANGE in *flags, so a
// damaged partition or COO cannot make the kernel touch other memory.
__global__ void __launch_bounds__(256)
    edge_spmv_kernel(const int32_t* __restrict__ ri, const int32_t* __restrict__ ci,
                     const float* __restrict__ val, const float* __restrict__ x,
                     float* __restrict__ y, long long rows, long long cols, long long nnz,
                     long long atoms, const int32_t* __restrict__ quarks,
                     const int32_t* __restrict__ atom_begin,
                     const int32_t* __restrict__ tile_begin, long long tiles,
                     int32_t* __restrict__ quark_tile, unsigned* __restrict__ flags) {
  constexpr unsigned kFull = 0xffffffffu;
  constexpr int kChunks = 4;
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  bool bad = false;
  for (long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < tiles;
       t += warps) {
    const long long a0 = min(max((long long)tile_begin[t], 0LL), atoms);
    const long long a1 = min(max((long long)tile_begin[t + 1], a0), atoms);
    const long long qb = min(max((long long)atom_begin[a0], 0LL), nnz);
    const long long qe = min(max((long long)atom_begin[a1], qb), nnz);
    // four 32-quark chunks per step, their loads issued together
    for (long long base = qb; base < qe; base += 32 * kChunks) {
      int q[kChunks], r[kChunks], c[kChunks];
      bool ok[kChunks];
      float v[kChunks], p[kChunks];
#pragma unroll
      for (int k = 0; k < kChunks; ++k) {
        const long long i = base + 32 * k + lane;
        ok[k] = i < qe;
        q[k] = ok[k] ? quarks[i] : 0;
        const bool in = (unsigned long long)(unsigned)q[k] < (unsigned long long)nnz;
        bad |= ok[k] && !in;
        ok[k] = ok[k] && in;
      }
#pragma unroll
      for (int k = 0; k < kChunks; ++k) {
        r[k] = ok[k] ? ri[q[k]] : 0;
        c[k] = ok[k] ? ci[q[k]] : 0;
        v[k] = ok[k] ? val[q[k]] : 0.f;
      }
#pragma unroll
      for (int k = 0; k < kChunks; ++k) {
        const bool in = (unsigned long long)(unsigned)r[k] < (unsigned long long)rows &&
                        (unsigned long long)(unsigned)c[k] < (unsigned long long)cols;
        bad |= ok[k] && !in;
        ok[k] = ok[k] && in;
        p[k] = ok[k] ? __fmul_rn(v[k], __ldg(x + c[k])) : 0.f;
        if (!ok[k]) r[k] = -1;
        if (ok[k] && quark_tile) quark_tile[q[k]] = (int32_t)t;
      }
#pragma unroll
      for (int k = 0; k < kChunks; ++k) {
        if (base + 32 * k >= qe) break;  // warp-uniform
        const int rp = __shfl_up_sync(kFull, r[k], 1);
        const unsigned heads = __ballot_sync(kFull, lane == 0 || rp != r[k]);
        const int start = 31 - __clz(heads & (kFull >> (31 - lane)));  // the run's first lane
        float s = p[k];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const float o = __shfl_up_sync(kFull, s, d);
          if (lane - d >= start) s += o;
        }
        const int rn = __shfl_down_sync(kFull, r[k], 1);
        if (ok[k] && (lane == 31 || rn != r[k])) atomicAdd(y + r[k], s);
      }
    }
  }
  if (bad) atomicOr(flags, EL_FLAG_INDEX_RANGE);
}

unsigned grid_for(long long n, int sms) {
  return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)sms * 8));
}

el_status sms_of_current(int* sms) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  *sms = device_info(device).sm_count;
  return EL_OK;
}

// the reference's argument rules [partitioner.hxx:85-93, :133-143]
el_status coordinate_grid(long long rows, long long cols, long long M0, long long K0,
                          long long M1, long long K1, Grid* g) {
  if (M0 <= 0 || K0 <= 0) return fail(EL_ERR_INVALID_ARGUMENT, "atom size must be > 0");
  if (M0 > rows || K0 > cols)
    return fail(EL_ERR_INVALID_ARGUMENT, "atom size %lld x %lld exceeds the matrix %lld x %lld",
                M0, K0, rows, cols);
  g->M0 = M0;
  g->K0 = K0;
  g->nax = (rows + M0 - 1) / M0;
  g->nay = (cols + K0 - 1) / K0;
  if (M1 <= 0 || K1 <= 0) return fail(EL_ERR_INVALID_ARGUMENT, "tile size must be > 0");
  if (M1 > g->nax || K1 > g->nay)
    return fail(EL_ERR_INVALID_ARGUMENT, "tile size %lld x %lld exceeds the atom grid %lld x %lld",
                M1, K1, g->nax, g->nay);
  g->M1 = M1;
  g->K1 = K1;
  g->ntx = (g->nax + M1 - 1) / M1;
  g->nty = (g->nay + K1 - 1) / K1;
  if (g->nax * g->nay >= (1LL << 31) - 1)
    return fail(EL_ERR_OVERFLOW, "%lld atoms exceed int32", g->nax * g->nay);
  return EL_OK;
}

el_status check_arrays(const el_edge_partition* P) {
  if (!P->atom_begin || !P->tile_begin || (P->nnz > 0 && !P->quarks) ||
      (P->num_atoms > 0 && (!P->atom_x || !P->atom_y)))
    return fail(EL_ERR_NULL_POINTER, "a partition array is NULL");
  return EL_OK;
}

}  // namespace
}  // namespace el

using namespace el;

extern "C" el_status el_edge_partition_coordinate_plan(int64_t rows, int64_t cols, int64_t nnz,
                                                       int64_t M0, int64_t K0, int64_t M1,
                                                       int64_t K1, el_edge_partition* P) {
  if (!P) return fail(EL_ERR_NULL_POINTER, "partition is NULL");
  if (rows < 0 || cols < 0 || nnz < 0) return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (nnz >= (1LL << 31) || rows >= (1LL << 31) || cols >= (1LL << 31))
    return fail(EL_ERR_OVERFLOW, "sizes exceed int32");
  Grid g;
  el_status st = coordinate_grid(rows, cols, M0, K0, M1, K1, &g);
  if (st != EL_OK) return st;
  P->nnz = nnz;
  P->num_atoms = g.nax * g.nay;
  P->num_tiles = g.ntx * g.nty;
  P->atoms_x = g.nax;
  P->atoms_y = g.nay;
  return EL_OK;
}

extern "C" el_status el_edge_partition_position_plan(int64_t nnz, int64_t nnz_per_atom,
                                                     int64_t atoms_per_tile,
                                                     el_edge_partition* P) {
  if (!P) return fail(EL_ERR_NULL_POINTER, "partition is NULL");
  if (nnz < 0) return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (nnz >= (1LL << 31)) return fail(EL_ERR_OVERFLOW, "nnz exceeds int32");
  // [partitioner.hxx:181-185]; a tile of no atoms is refused too
  if (nnz_per_atom <= 0) return fail(EL_ERR_INVALID_ARGUMENT, "nnz_per_atom must be > 0");
  if (nnz_per_atom > nnz)
    return fail(EL_ERR_INVALID_ARGUMENT, "nnz_per_atom %lld exceeds nnz %lld",
                (long long)nnz_per_atom, (long long)nnz);
  if (atoms_per_tile <= 0) return fail(EL_ERR_INVALID_ARGUMENT, "atoms_per_tile must be > 0");
  P->nnz = nnz;
  P->num_atoms = (nnz + nnz_per_atom - 1) / nnz_per_atom;
  P->num_tiles = (P->num_atoms + atoms_per_tile - 1) / atoms_per_tile;
  P->atoms_x = 0;
  P->atoms_y = 0;
  return EL_OK;
}

extern "C" el_status el_edge_partition_coordinate(el_workspace* ws, const el_coo* A, int64_t M0,
                                                  int64_t K0, int64_t M1, int64_t K1,
                                                  el_edge_partition* P, el_stream_t stream) {
  if (!A || !P) return fail(EL_ERR_NULL_POINTER, "matrix or partition is NULL");
  el_edge_partition want;
  el_status st = el_edge_partition_coordinate_plan(A->rows, A->cols, A->nnz, M0, K0, M1, K1,
                                                   &want);
  if (st != EL_OK) return st;
  if (P->nnz != want.nnz || P->num_atoms != want.num_atoms || P->num_tiles != want.num_tiles)
    return fail(EL_ERR_INVALID_ARGUMENT, "the partition was planned for other sizes");
  P->atoms_x = want.atoms_x;
  P->atoms_y = want.atoms_y;
  st = check_arrays(P);
  if (st != EL_OK) return st;
  const long long nnz = A->nnz;
  if (nnz > 0 && (!A->row_indices || !A->col_indices))
    return fail(EL_ERR_NULL_POINTER, "an index array is NULL");
  Grid g;
  coordinate_grid(A->rows, A->cols, M0, K0, M1, K1, &g);
  cudaStream_t s = (cudaStream_t)stream;
  int sms = 0;
  st = sms_of_current(&sms);
  if (st != EL_OK) return st;
  const long long atoms = want.num_atoms, tiles = want.num_tiles;
  unsigned long long* sorted = nullptr;
  if (nnz > 0) {
    // temporaries: keys in/out, positions in/out, the bad flag, CUB's storage
    const int end_bit = bits_for(atoms);
    size_t cub_bytes = 0;
    cub::DoubleBuffer<unsigned long long> kb(nullptr, nullptr);
    cub::DoubleBuffer<int32_t> pb(nullptr, nullptr);
    cudaError_t e =
        cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, kb, pb, (int)nnz, 0, end_bit, s);
    if (e != cudaSuccess) return cuda_status(e, "el_edge_partition_coordinate: sort size");
    const size_t kbytes = round256((size_t)nnz * 8), pbytes = round256((size_t)nnz * 4);
    const size_t total = 2 * kbytes + 2 * pbytes + 256 + round256(cub_bytes);
    el_workspace* w = nullptr;
    int device = 0;
    cudaGetDevice(&device);
    st = workspace_resolve(ws, s, device, &w);
    if (st != EL_OK) return st;
    void* stage = nullptr;
    cudaStream_t cs = nullptr;
    cudaEvent_t ev[4];
    st = workspace_stage(w, total, &stage, &cs, ev);
    if (st != EL_OK) return st;
    char* p = static_cast<char*>(stage);
    unsigned long long* k0 = reinterpret_cast<unsigned long long*>(p);
    unsigned long long* k1 = reinterpret_cast<unsigned long long*>(p + kbytes);
    int32_t* p0 = reinterpret_cast<int32_t*>(p + 2 * kbytes);
    int32_t* p1 = reinterpret_cast<int32_t*>(p + 2 * kbytes + pbytes);
    unsigned* bad = reinterpret_cast<unsigned*>(p + 2 * kbytes + 2 * pbytes);
    void* tmp = p + 2 * kbytes + 2 * pbytes + 256;
    e = cudaMemsetAsync(bad, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return cuda_status(e, "el_edge_partition_coordinate");
    rank_kernel<<<grid_for(nnz, sms), 256, 0, s>>>(A->row_indices, A->col_indices, nnz, A->rows,
                                                   A->cols, g, k0, p0, bad);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "el_edge_partition_coordinate: ranks");
    unsigned h_bad = 0;
    e = cudaMemcpyAsync(&h_bad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "el_edge_partition_coordinate: check");
    if (h_bad)
      return fail(EL_ERR_MALFORMED_CSR, "COO entry outside %lld x %lld", (long long)A->rows,
                  (long long)A->cols);
    cub::DoubleBuffer<unsigned long long> keys(k0, k1);
    cub::DoubleBuffer<int32_t> pos(p0, p1);
    size_t tb = round256(cub_bytes);
    e = cub::DeviceRadixSort::SortPairs(tmp, tb, keys, pos, (int)nnz, 0, end_bit, s);
    if (e != cudaSuccess) return cuda_status(e, "el_edge_partition_coordinate: sort");
    e = cudaMemcpyAsync(P->quarks, pos.Current(), (size_t)nnz * sizeof(int32_t),
                        cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_status(e, "el_edge_partition_coordinate: quarks");
    sorted = keys.Current();
  }
  atom_begin_kernel<<<grid_for(atoms + 1, sms), 256, 0, s>>>(sorted, nnz, atoms, P->atom_begin);
  if (atoms > 0)
    atom_coord_kernel<<<grid_for(atoms, sms), 256, 0, s>>>(g, atoms, P->atom_x, P->atom_y);
  tile_begin_kernel<<<grid_for(tiles + 1, sms), 256, 0, s>>>(g, tiles, atoms, P->tile_begin);
  return cuda_status(cudaGetLastError(), "el_edge_partition_coordinate");
}

extern "C" el_status el_edge_partition_position(int64_t nnz_per_atom, int64_t atoms_per_tile,
                                                el_edge_partition* P, el_stream_t stream) {
  if (!P) return fail(EL_ERR_NULL_POINTER, "partition is NULL");
  el_edge_partition want;
  el_status st = el_edge_partition_position_plan(P->nnz, nnz_per_atom, atoms_per_tile, &want);
  if (st != EL_OK) return st;
  if (P->num_atoms != want.num_atoms || P->num_tiles != want.num_tiles)
    return fail(EL_ERR_INVALID_ARGUMENT, "the partition was planned for other sizes");
  P->atoms_x = P->atoms_y = 0;
  st = check_arrays(P);
  if (st != EL_OK) return st;
  int sms = 0;
  st = sms_of_current(&sms);
  if (st != EL_OK) return st;
  const long long n = std::max<long long>(P->nnz, P->num_atoms + 1);
  position_kernel<<<grid_for(n, sms), 256, 0, (cudaStream_t)stream>>>(
      P->nnz, nnz_per_atom, P->num_atoms, atoms_per_tile, P->num_tiles, P->quarks,
      P->atom_begin, P->atom_x, P->atom_y, P->tile_begin);
  return cuda_status(cudaGetLastError(), "el_edge_partition_position");
}

extern "C" el_status el_spmv_edge(el_workspace* ws, const el_coo* A, const el_edge_partition* P,
                                  const float* x, float* y, int32_t* quark_tile,
                                  el_stream_t stream) {
  if (!A || !P) return fail(EL_ERR_NULL_POINTER, "matrix or partition is NULL");
  if (A->rows < 0 || A->cols < 0 || A->nnz < 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (P->nnz != A->nnz) return fail(EL_ERR_INVALID_ARGUMENT, "partition of another matrix");
  if (A->rows > 0 && !y) return fail(EL_ERR_NULL_POINTER, "y is NULL");
  if (A->nnz > 0 && (!A->row_indices || !A->col_indices || !A->values || !x))
    return fail(EL_ERR_NULL_POINTER, "an input array is NULL");
  el_status st = check_arrays(P);
  if (st != EL_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (A->rows > 0) {
    cudaError_t e = cudaMemsetAsync(y, 0, (size_t)A->rows * sizeof(float), s);
    if (e != cudaSuccess) return cuda_status(e, "el_spmv_edge: y");
  }
  if (P->num_tiles == 0 || A->nnz == 0) return EL_OK;
  int sms = 0, device = 0;
  st = sms_of_current(&sms);
  if (st != EL_OK) return st;
  cudaGetDevice(&device);
  el_workspace* w = nullptr;
  st = workspace_resolve(ws, s, device, &w);
  if (st != EL_OK) return st;
  unsigned* flags = &workspace_view(w).hdr->errors;
  // a warp per tile, 8 per block
  const long long blocks = std::min<long long>((P->num_tiles + 7) / 8, (long long)sms * 8);
  edge_spmv_kernel<<<(unsigned)blocks, 256, 0, s>>>(
      A->row_indices, A->col_indices, A->values, x, y, A->rows, A->cols, A->nnz, P->num_atoms,
      P->quarks, P->atom_begin, P->tile_begin, P->num_tiles, quark_tile, flags);
  return cuda_status(cudaGetLastError(), "el_spmv_edge");
}

extern "C" el_status el_coo_sort(el_workspace* ws, el_coo* A, int32_t by_column,
                                 el_stream_t stream) {
  if (!A) return fail(EL_ERR_NULL_POINTER, "matrix is NULL");
  if (A->rows < 0 || A->cols < 0 || A->nnz < 0)
    return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (A->rows >= (1LL << 31) || A->cols >= (1LL << 31) || A->nnz >= (1LL << 31))
    return fail(EL_ERR_OVERFLOW, "sizes exceed int32");
  if (by_column != 0 && by_column != 1)
    return fail(EL_ERR_INVALID_ARGUMENT, "by_column must be 0 or 1");
  const long long nnz = A->nnz;
  if (nnz == 0) return EL_OK;
  if (!A->row_indices || !A->col_indices || !A->values)
    return fail(EL_ERR_NULL_POINTER, "an array is NULL");
  cudaStream_t s = (cudaStream_t)stream;
  int sms = 0;
  el_status st = sms_of_current(&sms);
  if (st != EL_OK) return st;
  const long long major = by_column ? A->cols : A->rows;
  const int end_bit = 31 + bits_for(major > 0 ? major : 1);
  size_t cub_bytes = 0;
  cub::DoubleBuffer<unsigned long long> kb(nullptr, nullptr);
  cub::DoubleBuffer<int32_t> pb(nullptr, nullptr);
  cudaError_t e =
      cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, kb, pb, (int)nnz, 0, end_bit, s);
  if (e != cudaSuccess) return cuda_status(e, "el_coo_sort: sort size");
  // temporaries: keys in/out, positions in/out, a copy of the values, the
  // bad flag, CUB's storage
  const size_t kbytes = round256((size_t)nnz * 8), pbytes = round256((size_t)nnz * 4);
  const size_t total = 2 * kbytes + 3 * pbytes + 256 + round256(cub_bytes);
  el_workspace* w = nullptr;
  int device = 0;
  cudaGetDevice(&device);
  st = workspace_resolve(ws, s, device, &w);
  if (st != EL_OK) return st;
  void* stage = nullptr;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev[4];
  st = workspace_stage(w, total, &stage, &cs, ev);
  if (st != EL_OK) return st;
  char* p = static_cast<char*>(stage);
  unsigned long long* k0 = reinterpret_cast<unsigned long long*>(p);
  unsigned long long* k1 = reinterpret_cast<unsigned long long*>(p + kbytes);
  int32_t* p0 = reinterpret_cast<int32_t*>(p + 2 * kbytes);
  int32_t* p1 = reinterpret_cast<int32_t*>(p + 2 * kbytes + pbytes);
  float* vcopy = reinterpret_cast<float*>(p + 2 * kbytes + 2 * pbytes);
  unsigned* bad = reinterpret_cast<unsigned*>(p + 2 * kbytes + 3 * pbytes);
  void* tmp = p + 2 * kbytes + 3 * pbytes + 256;
  e = cudaMemsetAsync(bad, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return cuda_status(e, "el_coo_sort");
  coo_keys_kernel<<<grid_for(nnz, sms), 256, 0, s>>>(A->row_indices, A->col_indices, nnz, A->rows,
                                                     A->cols, by_column, k0, p0, bad);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "el_coo_sort: keys");
  unsigned h_bad = 0;
  e = cudaMemcpyAsync(&h_bad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "el_coo_sort: check");
  if (h_bad)
    return fail(EL_ERR_MALFORMED_CSR, "COO entry outside %lld x %lld", (long long)A->rows,
                (long long)A->cols);
  cub::DoubleBuffer<unsigned long long> keys(k0, k1);
  cub::DoubleBuffer<int32_t> pos(p0, p1);
  size_t tb = round256(cub_bytes);
  e = cub::DeviceRadixSort::SortPairs(tmp, tb, keys, pos, (int)nnz, 0, end_bit, s);
  if (e != cudaSuccess) return cuda_status(e, "el_coo_sort: sort");
  e = cudaMemcpyAsync(vcopy, A->values, (size_t)nnz * sizeof(float), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "el_coo_sort: values");
  coo_scatter_kernel<<<grid_for(nnz, sms), 256, 0, s>>>(keys.Current(), pos.Current(), vcopy, nnz,
                                                        by_column, A->row_indices,
                                                        A->col_indices, A->values);
  return cuda_status(cudaGetLastError(), "el_coo_sort: scatter");
}

extern "C" el_status el_csr_row_indices(const int32_t* offsets, int64_t rows, int64_t nnz,
                                        int32_t* row_indices, el_stream_t stream) {
  if (rows < 0 || nnz < 0) return fail(EL_ERR_INVALID_ARGUMENT, "negative size");
  if (rows >= (1LL << 31) || nnz >= (1LL << 31)) return fail(EL_ERR_OVERFLOW, "sizes exceed int32");
  if (rows == 0 || nnz == 0) return EL_OK;
  if (!offsets || !row_indices) return fail(EL_ERR_NULL_POINTER, "an array is NULL");
  int sms = 0;
  el_status st = sms_of_current(&sms);
  if (st != EL_OK) return st;
  // a warp per row: 8 rows per block of 256
  const long long blocks = std::min<long long>((rows + 7) / 8, (long long)sms * 16);
  row_indices_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(offsets, rows,
                                                                          row_indices);
  return cuda_status(cudaGetLastError(), "el_csr_row_indices");
}
